#!/usr/bin/env python3
"""Benchmark: MAC-Poisson time to a 1e-8 relative residual and leaf cells/s on
one GB300.  Default workload: the largest single-GPU configuration, the batch
of 256 independent 2D problems (64-1024 leaf blocks of 16x16 cells each, 1-4
ellipse IB solids, rho ratio 10-1000; 29.4M leaf cells) solved as one forest;
--config selects the others (config2: 2D 6 levels, config3: 3D 16^3 blocks,
config5: the elbow pipe).

A step is one complete MG-preconditioned BiCGSTAB solve from a zero initial
guess to |r|_inf < 1e-8 |r0|_inf (the reference's criterion,
src/SayakaMacSolver.cpp:891).

  value : leaf cells / device time of a solve, inputs resident in HBM,
          L2 flushed (256 MiB write) before every timed solve; N replicas
          under torchrun add up (replicas only: one tree per GPU)
  e2e   : the same through the C ABI with host buffers in the reference's
          TreeData layout (setRhs -> cg_solve -> getSol per step)
  cpu_baseline / --impl reference : the C oracle (bit-exact restatement of
          the reference solver) on the host cores, bounded sample (for the
          batch workload: whole problems of the batch, one per core).
  solvers : time to 1e-8 of plain FP64 MG-BiCGSTAB, of the FP32 V-cycle and
          of the learned correction with the FP32 V-cycle, same workload.
  error_vs_oracle : relative L2 over fluid leaf cells of the device solution
          against the C oracle's converged FP64 solve (the batch workload:
          its first problems), and the final true residual.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MAC Poisson time to 1e-8 rel residual & cells/s: learned+FP32 vs plain MG, GB300"
TOL = 1e-8
# iteration limit of a solver setting tried by the setting search
TUNE_MAX_ITER = 200
# CPU reference solve: the reference algorithm with its bottom BiCGSTAB run
# to convergence (relative 1e-10) -- the preconditioner the GPU path applies
# exactly.  With the reference's default bottom tolerances (1e-6 relative and
# absolute) its outer BiCGSTAB does not reach 1e-8 on this workload within
# 2000 iterations (the bottom tolerance becomes absolute as the residual
# falls; see the design notes).
CPU_BOTTOM_TOL = 1e-10
WORKLOADS = {
    "config1": "unit square, 4x4 roots, circle r=0.25 refinement, B=1, Neumann walls",
    "config2": "rho 1:1000 across a smoothed ellipse, fractional IB disk (faces beside solid cells closed), "
               "p=0 top wall",
    "config3": "sphere r=0.2 refinement band, IB sphere mask, B ratio 100 across a blob, p=0 top wall",
    "config4": "256 independent problems (64-1024 leaf blocks, 1-4 ellipse IB solids, rho ratio 10-1000) "
               "solved as one forest",
    "config5": "90-degree elbow pipe (tube 0.1, bend 0.3) with a sphere inside as IB, p=0 outlet, first solve "
               "of the regrid sequence",
}
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="config4")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain-FP64 / FP32 / learned comparison and the oracle error")
    ap.add_argument("--precision", type=int, default=-1,
                    help="V-cycle precision: 1 FP32, 0 FP64, -1 (default) the faster of the two, timed during "
                         "warm-up (the outer BiCGSTAB and its 1e-8 test are FP64 either way)")
    ap.add_argument("--n-post", type=int, default=-1,
                    help="post-smoothing sweeps per level (the reference's setPostSmoothNum, its default 2); "
                         "-1 (default): 1 or 2, whichever solves faster in the warm-up timing")
    ap.add_argument("--smoother", type=int, default=-1,
                    help="V-cycle smoother: 0 red-black sweeps (one launch per colour), 1 block-hybrid passes "
                         "(Gauss-Seidel inside a block, Jacobi between blocks); -1 (default): timed during warm-up")
    ap.add_argument("--inner-sweeps", type=int, default=-1,
                    help="smoother 1: red-black sweeps per block and pass (-1: 2 or 3, timed during warm-up)")
    ap.add_argument("--pdl", type=int, default=0, help="programmatic dependent launch between kernels")
    ap.add_argument("--vcycle-kernel", type=int, default=0,
                    help="0: one launch per phase, 1: whole V-cycle as one cooperative launch, "
                         "2: runs of small phases inside one thread-block cluster")
    ap.add_argument("--cluster-cells", type=int, default=16384,
                    help="vcycle-kernel 2: largest phase (cells) that runs inside the cluster")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--bottom-level", type=int, default=0,
                    help="level of the dense bottom solve (0: the coarsest uniform level of at most 4096 cells "
                         "per component)")
    ap.add_argument("--bottom-half", type=int, default=0,
                    help="1: FP16 copy of the dense bottom inverse (bottom level above 1)")
    ap.add_argument("--sublevel-order", type=int, default=1,
                    help="V-cycle smoothing order over a tower's sublevels: 0 finest to coarsest per sublevel "
                         "(the reference's), 1 one launch per colour and level parity")
    ap.add_argument("--smooth-variant", type=int, default=-1,
                    help="device smoother launch-bounds variant (-1: autotuned at prepare)")
    ap.add_argument("--omega", type=float, default=-1.0,
                    help="relaxation weight of the V-cycle's red-black updates (params.relax_omega; -1: 1.0, 1.1 or "
                         "1.2, timed during warm-up with the chosen setting)")
    ap.add_argument("--vcycle-out", type=int, default=0,
                    help="FP32 V-cycle output: 0 auto (in place in 2D and on small 3D towers), 1 in place with the "
                         "operator in double-float, 2 widened into FP64 vectors, 3 in place")
    ap.add_argument("--kernel", type=int, default=-1,
                    help="time one kernel alone and exit (for ncu): 0 FP64 operator on the finest tower, "
                         "1 FP32 / 2 FP64 red-black sweep (one colour) of the finest level, "
                         "3 the device solve's FP64 operator + dot product")
    ap.add_argument("--sequence", type=int, default=0,
                    help="config5 only: time a sequence of this many pressure solves of the elbow with the sphere "
                         "moving along the pipe, a regrid every --regrid-every steps, setup inside the timed region")
    ap.add_argument("--regrid-every", type=int, default=5)
    ap.add_argument("--problems", type=int, default=256,
                    help="config4: number of problems of the batch (256; fewer for a small profiling case)")
    ap.add_argument("--max-level", type=int, default=7, help="--sequence: finest level of the elbow tree")
    ap.add_argument("--bottom-refresh", type=int, default=0,
                    help="--sequence: 1 rebuild the dense bottom inverse after every coefficient change, 0 (default) "
                         "keep the inverse of the last tree between regrids")
    ap.add_argument("--transfer", default="centered_linear", choices=["centered_linear", "injection"],
                    help="--sequence: the solution carried across a regrid by the reference's transfer "
                         "(average-down, centered-linear new blocks; default) or by injection")
    ap.add_argument("--profile", action="store_true",
                    help="run one solve between cudaProfilerStart/Stop (for ncu --profile-from-start off) and exit")
    return ap.parse_args()


def max_over_ranks(x, ws, device):
    """the slowest rank's time: every replica's solve must be done"""
    if ws <= 1:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(cells_per_rank, ws, ms_step):
    """whole-job cells/s: ws replicas of the workload in the slowest rank's time"""
    return ws * cells_per_rank / (ms_step / 1e3)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region"""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def treedata_cell_buffer(prob, cells, ngrow=1):
    """compact cells -> the reference's TreeData layout (1 component, ngrow ghosts)"""
    nd, nb, n = prob.ndim, prob.nb, prob.num_blocks
    G = nb + 2 * ngrow
    shape = (n,) + (G,) * nd
    buf = np.zeros(shape)
    inner = (slice(None),) + (slice(ngrow, ngrow + nb),) * nd
    buf[inner] = cells.reshape((n,) + (nb,) * nd)
    return buf.reshape(-1)


def cpu_oracle(prob):
    from oracle import pyoracle
    vf, af, bc = pyoracle.setup_coefficients(prob.tables, prob.bc, prob.vol, prob.area, prob.bface)
    return pyoracle, pyoracle.Oracle(prob.tables, prob.bc, vf, af, bc)


# above this many leaf cells the CPU legs time a bounded sample of outer
# iterations instead of a full solve (a full one-thread solve of the 3D and
# batch workloads takes from minutes to hours)
CPU_FULL_CELLS = 1_000_000
CPU_SAMPLE_S = 20.0


def cpu_solve(prob, max_iter=2000, budget_s=None, n_iters=None):
    """the oracle's reference solver on one host thread.  Without a budget:
    a full solve to 1e-8.  With one: 1 outer iteration, then k iterations
    sized to the budget; seconds per iteration = (t_k - t_1) / (k - 1) (the
    setup excluded; k >= 3), and the iterations to 1e-8 are the
    solve's own when it converged within k, else n_iters when given (the
    device solve's count on the same workload), else extrapolated from the
    residual reduction observed over the k iterations (rough: BiCGSTAB's
    early reduction is not geometric).  The reference's outer iterations get
    dearer as the solve proceeds (its bottom BiCGSTAB works harder as the
    outer residual falls), so the sampled rate overstates the CPU's: the
    bounded baseline favours the CPU."""
    pyoracle, O = cpu_oracle(prob)

    def run(n):
        t0 = time.perf_counter()
        _, info = O.cg_solve(prob.rhs, pyoracle.params(max_iter=n, tol_rel=TOL, tol_abs=0.0,
                                                       bot_tol_rel=CPU_BOTTOM_TOL, bot_tol_abs=0.0))
        return time.perf_counter() - t0, info

    if budget_s is None:
        dt, info = run(max_iter)
        return dict(seconds=dt, iterations=info["iterations"], status=info["status"], value=prob.leaf_cells / dt,
                    sampled=False, per_iteration=dt / max(1, info["iterations"]))
    t1, _ = run(1)
    tk, info = run(int(max(3, min(max_iter, budget_s / t1))))
    per_it = (tk - t1) / (info["iterations"] - 1) if info["iterations"] > 1 else tk
    if info["status"] == 0:
        n_it = info["iterations"]
    elif n_iters:
        n_it = int(n_iters)
    else:
        red = info["rnorm"] / info["rnorm0"] if info["rnorm0"] > 0 else float("nan")
        n_it = int(math.ceil(info["iterations"] * math.log(TOL) / math.log(red))) if 0 < red < 1 else 0
    if n_it <= 0:
        return dict(seconds=float("nan"), iterations=0, status=2, value=float("nan"), sampled=True,
                    per_iteration=per_it, sample_iterations=info["iterations"])
    return dict(seconds=per_it * n_it, iterations=n_it, status=0, value=prob.leaf_cells / (per_it * n_it),
                sampled=True, per_iteration=per_it, sample_iterations=info["iterations"])


def oracle_workloads():
    """the workload generators with their trees built by the oracle's
    restatement of the reference's tree (oracle/tree_oracle.py, the same
    tables bit for bit), so that the reference arm runs no product code"""
    from sayakaamr_gb300 import workloads
    from oracle.tree_oracle import TreeOracle
    workloads.use_tree_builder(TreeOracle)
    return workloads


def _cpu_worker(args):
    name, max_iter, budget = args
    workloads = oracle_workloads()
    prob = workloads.CONFIGS[name]()
    return cpu_solve(prob, max_iter, budget)


def cpu_payload(p):
    """a problem without its tree handle (picklable for the worker processes)"""
    from sayakaamr_gb300 import workloads
    q = workloads.Problem(p.name, None, p.tables, p.bc, p.vol, p.area, p.bface, p.rhs, p.params)
    return q


def _cpu_part_worker(q):
    """one whole problem of the batch solved to 1e-8 by the oracle"""
    return cpu_solve(q)


def cpu_batch_sample(parts, budget_s=CPU_SAMPLE_S):
    """the batch workload on one host thread: its problems solved whole, one
    after another, until about budget_s seconds have passed"""
    cells = secs = 0.0
    its = []
    k = 0
    for p in parts:
        r = cpu_solve(p)
        if r["status"] != 0:
            raise SystemExit("CPU reference solve of %s did not converge" % p.name)
        cells += p.leaf_cells
        secs += r["seconds"]
        its.append(r["iterations"])
        k += 1
        if secs >= budget_s:
            break
    return dict(value=cells / secs, problems=k, cells=int(cells), seconds=secs, iterations=its)


def run_reference(args):
    """--impl reference: the reference solver (the C oracle port: the
    reference library itself does not travel to the GPU host) on every host
    core, one copy of the workload per core.  The first round is a full solve
    per core (iterations to 1e-8 and seconds per iteration); every step is a
    bounded sample of outer iterations per core, and its value is
    cores x leaf cells / (seconds per iteration x iterations to 1e-8)."""
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import multiprocessing as mp
    workloads = oracle_workloads()
    prob = (workloads.config4(n_problems=args.problems) if args.config == "config4"
            else workloads.CONFIGS[args.config]())
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    if getattr(prob, "parts", None):
        run_reference_batch(args, prob, cores, ctx)
        return
    t_all = time.perf_counter()
    with ctx.Pool(cores) as pool:
        big = prob.leaf_cells > CPU_FULL_CELLS
        full = pool.map(_cpu_worker, [(args.config, 2000, CPU_SAMPLE_S if big else None)] * cores)
        if any(r["status"] != 0 for r in full):
            print(json.dumps({"impl": "reference", "unavailable": "CPU reference solve did not converge"}))
            return
        n_it = full[0]["iterations"]
        per_it = statistics.mean(r["per_iteration"] for r in full)
        # bounded steps: about 60 s of sampling in total
        k_it = int(max(1, min(n_it, 60.0 / max(1, args.steps + args.warmup) / per_it)))
        vals = []
        for s in range(args.warmup + args.steps):
            if big:  # the first round's sample stands for every step
                res = full
            else:
                res = pool.map(_cpu_worker, [(args.config, k_it, None)] * cores)
            if s >= args.warmup:
                vals.append(sum(prob.leaf_cells / (r["per_iteration"] * n_it) for r in res))
    wall = time.perf_counter() - t_all
    v = statistics.mean(vals)
    ms = prob.leaf_cells / (v / cores) * 1e3
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.config, **prob.describe(), "tol_rel": TOL,
                   "trees": "built by the oracle's restatement of the reference's tree (oracle/tree_oracle.py)"},
        "cpu_baseline": {"value": v, "unit": "cells/s", "cores": cores, "kind": "port",
                         "sample": ("C oracle (bit-exact restatement of the reference solver, bottom BiCGSTAB to "
                                    "1e-10), one copy of the workload per core; " +
                                    ("a bounded sample per core (%d outer iterations, %.3f s each; %d iterations "
                                     "to 1e-8 extrapolated from its residual reduction)"
                                     % (full[0]["sample_iterations"], per_it, n_it) if big else
                                     "full solve per core first (%d outer iterations to 1e-8, %.3f s each), then "
                                     "%d-iteration samples per step" % (n_it, per_it, k_it)))},
        "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(out))


def run_reference_batch(args, prob, cores, ctx):
    """--impl reference on the batch workload: every step solves `cores`
    whole problems of the batch (consecutive ones, wrapping around) on all
    host cores at once, one problem per core, each to 1e-8 by the oracle;
    value = their leaf cells / the step's wall time"""
    parts = [cpu_payload(p) for p in prob.parts]
    t_all = time.perf_counter()
    vals, its = [], []
    k0 = 0
    with ctx.Pool(cores) as pool:
        for s in range(args.warmup + args.steps):
            chunk = [parts[(k0 + i) % len(parts)] for i in range(cores)]
            k0 += cores
            t0 = time.perf_counter()
            res = pool.map(_cpu_part_worker, chunk)
            dt = time.perf_counter() - t0
            if any(r["status"] != 0 for r in res):
                print(json.dumps({"impl": "reference", "unavailable": "CPU reference solve did not converge"}))
                return
            if s >= args.warmup:
                vals.append(sum(q.leaf_cells for q in chunk) / dt)
                its.extend(r["iterations"] for r in res)
    wall = time.perf_counter() - t_all
    v = statistics.mean(vals)
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": prob.leaf_cells / v * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.config, **prob.describe(), "tol_rel": TOL,
                   "trees": "built by the oracle's restatement of the reference's tree (oracle/tree_oracle.py)"},
        "cpu_baseline": {"value": v, "unit": "cells/s", "cores": cores, "kind": "port",
                         "sample": ("C oracle (bit-exact restatement of the reference solver, bottom BiCGSTAB to "
                                    "1e-10); each step solves %d whole problems of the batch to 1e-8, one per "
                                    "core (%d problem solves timed, %.1f outer iterations on average); "
                                    "ms_per_step = the whole batch's leaf cells at that rate"
                                    % (cores, len(its), statistics.mean(its)))},
        "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(out))


def fluid_leaf_rel_error(p, vf, sol, ref):
    nc = p.ncell
    m = vf.reshape(-1, nc)[p.leaf].reshape(-1) > 0
    a = sol.reshape(-1, nc)[p.leaf].reshape(-1)[m]
    b = ref.reshape(-1, nc)[p.leaf].reshape(-1)[m]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


ORACLE_PROBLEMS = 4  # batch workload: problems compared with the oracle


def oracle_check(S, prob, timed_sol):
    """the device solution against the oracle's converged FP64 solve (tol
    1e-11, bottom 1e-10): at the timed tolerance (1e-8, the solution of the
    last timed solve) and after a solve to 1e-11; the batch workload on its
    first ORACLE_PROBLEMS problems.  Also the final true residual of the timed
    solution under the reference-arithmetic operator, max over fluid leaf
    cells relative to the right-hand side's."""
    from oracle import pyoracle
    parts = getattr(prob, "parts", None)
    if not parts and prob.leaf_cells > 2 * CPU_FULL_CELLS:
        return {"skipped": "a converged oracle solve of %d cells takes longer than the bench's CPU budget; "
                           "tests/test_gpu_workload_parity.py compares the device solve with the oracle on a "
                           "reduced tree of this geometry" % prob.leaf_cells}
    checks = [(p, prob.block_offsets[k]) for k, p in enumerate(parts[:ORACLE_PROBLEMS])] if parts else [(prob, 0)]
    # true residual of the timed solution (reference-arithmetic kernel)
    finest = int(prob.tables["level"].max())
    r = S.residual(finest, timed_sol, prob.rhs)
    vf_all = S.get_coef(2)
    leafm = np.zeros(prob.num_blocks, dtype=bool)
    leafm[prob.leaf] = True
    fl = (vf_all.reshape(-1, prob.ncell) > 0) & leafm[:, None]
    true_res = float(np.abs(r.reshape(-1, prob.ncell)[fl]).max() / np.abs(prob.rhs.reshape(-1, prob.ncell)[fl]).max())
    S.set_params(tol_rel=1e-11)
    S.prepare()
    S.set_zero_sol()
    info = S.cg_solve()
    tight = S.get_sol_compact()
    S.set_params(tol_rel=TOL)
    S.prepare()
    e8, e11 = [], []
    t0 = time.perf_counter()
    for p, b0 in checks:
        vf, af, bc = pyoracle.setup_coefficients(p.tables, p.bc, p.vol, p.area, p.bface)
        O = pyoracle.Oracle(p.tables, p.bc, vf, af, bc)
        ref, oinfo = O.cg_solve(p.rhs, pyoracle.params(tol_rel=1e-11, tol_abs=0.0, bot_tol_rel=1e-10,
                                                       bot_tol_abs=0.0))
        if oinfo["status"] != 0:
            raise SystemExit("oracle solve of %s did not converge" % p.name)
        sl = slice(b0 * p.ncell, (b0 + p.num_blocks) * p.ncell)
        e8.append(fluid_leaf_rel_error(p, vf, timed_sol[sl], ref))
        e11.append(fluid_leaf_rel_error(p, vf, tight[sl], ref))
    return {"at_1e-8": max(e8), "at_1e-11": max(e11),
            "true_residual_rel_inf": true_res,
            "device_rnorm_rel_at_1e-11": info["rnorm"] / info["rnorm0"] if info["rnorm0"] else 0.0,
            "sample": ("%s; relative L2 over fluid leaf cells against the C oracle's FP64 solve to 1e-11 "
                       "(bottom BiCGSTAB to 1e-10), max over the problems; oracle time %.1f s"
                       % ("the batch's first %d problems" % len(checks) if parts else "the whole workload",
                          time.perf_counter() - t0))}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    ws, rank, local = dist_info()
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import sayakaamr_gb300 as sg
    from sayakaamr_gb300 import workloads

    if args.sequence > 0:
        run_sequence(args, torch, ws, rank, local)
        return
    prob = (workloads.config4(n_problems=args.problems) if args.config == "config4"
            else workloads.CONFIGS[args.config]())
    S = workloads.make_solver(prob)
    S.set_params(tol_rel=TOL, tol_abs=0.0, use_mg_precond=1, max_iter=2000, precision=max(args.precision, 0),
                 bottom=1,
                 graph=0 if args.profile else 1, n_post_smooth=max(args.n_post, 1) if args.n_post >= 0 else 2,
                 vcycle_kernel=args.vcycle_kernel,
                 cluster_cells=args.cluster_cells, smooth_variant=args.smooth_variant, vcycle_out=args.vcycle_out,
                 pdl=args.pdl, sublevel_order=args.sublevel_order, bottom_level=args.bottom_level,
                 bottom_half=args.bottom_half, smoother=max(args.smoother, 0),
                 inner_sweeps=args.inner_sweeps if args.inner_sweeps > 0 else 2,
                 relax_omega=args.omega if args.omega > 0 else 1.0)
    S.prepare()
    ext = torch.cuda.ExternalStream(S.stream())
    if args.kernel >= 0:
        kernel_only(S, prob, ext, torch, args)
        return
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    finest = int(prob.tables["level"].max())

    def one(timed_events=None):
        with torch.cuda.stream(ext):
            flush.zero_()
        if timed_events:
            timed_events[0].record(ext)
        S.set_zero_sol()
        S.cg_solve_async()
        if timed_events:
            timed_events[1].record(ext)
        return S.solve_info()

    def warm(setting=None, ok=(0,), tolerate=False):
        """W warm-up solves; a failed one ends the run, or (tolerate) is
        returned as a description"""
        for _ in range(args.warmup):
            info = one()
            if info["status"] not in ok:
                st = S.problem_states()
                where = ""
                if st is not None:
                    its, rel = st
                    bad = [(int(i), int(its[i]), float(rel[i])) for i in range(len(rel)) if not rel[i] < TOL]
                    where = "; problems not converged (index, iterations, relative residual): %s" % bad[:8]
                msg = "warm-up solve failed: %s, setting %s%s" % (info, setting, where)
                if tolerate:
                    return msg
                raise SystemExit(msg)
        return None

    tuning = None
    if args.precision < 0 or args.n_post < 0 or args.smoother < 0:
        # the faster solver setting on this workload, from timed warm-up
        # solves: V-cycle precision (FP32 / FP64), smoother (red-black sweeps
        # or block-hybrid passes of inner_sweeps sweeps) and post-smoothing
        # sweeps / passes per tower
        tuning = []
        precs = (1, 0) if args.precision < 0 else (args.precision,)
        smoothers = (0, 1) if args.smoother < 0 else (args.smoother,)
        families = []
        for prec in precs:
            for sm in smoothers:
                if sm == 0:
                    families.append((prec, 0, 2, (1, 2, 3, 4, 6, 8)))
                else:
                    for inner in ((2, 3) if args.inner_sweeps < 0 else (args.inner_sweeps,)):
                        families.append((prec, 1, inner, (1, 2, 3, 4)))
        for prec, sm, inner, posts in families:
            # more sweeps trade V-cycle cost for iterations: 2D latency-bound
            # solves prefer 2, 3D ones 3-4; the search over a family stops
            # after two settings slower than its best
            if args.n_post >= 0:
                posts = (args.n_post,)
            best_f, worse = None, 0
            for npost in posts:
                # a setting that needs more than TUNE_MAX_ITER iterations is
                # not a candidate: it is recorded as not converged and skipped
                S.set_params(precision=prec, n_post_smooth=npost, smoother=sm, inner_sweeps=inner,
                             max_iter=TUNE_MAX_ITER)
                S.prepare()
                failed = warm(dict(precision=prec, smoother=sm, inner_sweeps=inner, n_post_smooth=npost),
                              tolerate=True)
                if failed:
                    tuning.append(dict(precision=prec, smoother=sm, inner_sweeps=inner, n_post_smooth=npost,
                                       ms=None, not_converged=failed[:300]))
                    worse += 1
                    if worse >= 2:
                        break
                    continue
                ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
                infos = [one(e) for e in ev]
                torch.cuda.synchronize()
                t = statistics.mean(a.elapsed_time(b) for a, b in ev)
                tuning.append(dict(precision=prec, smoother=sm, inner_sweeps=inner, n_post_smooth=npost, ms=t,
                                   iterations=statistics.mean(i["iterations"] for i in infos)))
                if best_f is None or t < best_f:
                    best_f, worse = t, 0
                else:
                    worse += 1
                    if worse >= 2:
                        break
        best = min((r for r in tuning if r["ms"] is not None), key=lambda r: r["ms"])
        args.precision, args.n_post = best["precision"], best["n_post_smooth"]
        args.smoother, args.inner_sweeps = best["smoother"], best["inner_sweeps"]
        S.set_params(precision=args.precision, n_post_smooth=args.n_post, smoother=args.smoother,
                     inner_sweeps=args.inner_sweeps, max_iter=2000)
        S.prepare()
    if args.inner_sweeps < 0:
        args.inner_sweeps = 2
    omega_tuning = None
    if args.omega < 0:
        # the smoother's relaxation weight with the chosen setting, timed the
        # same way: over-relaxed red-black sweeps are another fixed linear
        # preconditioner (the same solution), often with fewer iterations
        omega_tuning = []
        for om in (1.0, 1.1, 1.2):
            S.set_params(relax_omega=om, max_iter=TUNE_MAX_ITER)
            S.prepare()
            failed = warm(dict(relax_omega=om), tolerate=True)
            if failed:
                omega_tuning.append(dict(omega=om, ms=None, not_converged=failed[:300]))
                continue
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
            infos = [one(e) for e in ev]
            torch.cuda.synchronize()
            omega_tuning.append(dict(omega=om, ms=statistics.mean(a.elapsed_time(b) for a, b in ev),
                                     iterations=statistics.mean(i["iterations"] for i in infos)))
        args.omega = min((r for r in omega_tuning if r["ms"] is not None), key=lambda r: r["ms"])["omega"]
    S.set_params(relax_omega=args.omega, max_iter=2000)
    S.prepare()
    warm()
    if args.profile:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        info = one()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"profiled_solve": info, "launches_per_iteration": S.launch_counts()[1]}))
        return
    pro, per_it, epi = S.launch_counts()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    infos = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            infos.append(one(events[k]))
        torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ms = [a.elapsed_time(b) for a, b in events]
    ms_step = statistics.mean(ms)
    ms_step = max_over_ranks(ms_step, ws, "cuda")
    bad = [i for i in infos if i["status"] != 0 or not (i["rnorm"] < TOL * i["rnorm0"])]
    if bad:
        raise SystemExit("timed solve did not converge: %s" % bad[0])
    iters = [i["iterations"] for i in infos]
    value = job_value(prob.leaf_cells, ws, ms_step)
    launches = int(round(statistics.mean(pro + it * per_it + epi for it in iters)))

    # ---- end to end through the C ABI with host TreeData buffers ----
    rhs_td = treedata_cell_buffer(prob, prob.rhs, ngrow=1)
    sol_td = np.zeros_like(rhs_td)
    import ctypes
    pin_rhs = torch.from_numpy(rhs_td).pin_memory()
    pin_sol = torch.from_numpy(sol_td).pin_memory()
    rhs_np = pin_rhs.numpy()
    sol_np = pin_sol.numpy()
    e2e_t = []
    for k in range(0 if args.no_e2e else args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        S.set_rhs(rhs_np, ncomp=1, ngrow=1, comp=0)
        S.set_zero_sol()
        info = S.cg_solve()
        S.get_sol(sol_np, ncomp=1, ngrow=1, comp=0)
        t1 = time.perf_counter()
        if info["status"] != 0:
            raise SystemExit("e2e solve failed: %s" % info)
        if k >= args.warmup:
            e2e_t.append(t1 - t0)
    e2e_s = statistics.mean(e2e_t) if e2e_t else float("nan")
    h2d = prob.num_blocks * prob.ncell * 8
    d2h = prob.num_blocks * prob.ncell * 8

    # ---- the metric's comparison: plain FP64 MG vs the FP32 V-cycle vs the
    # learned correction with the FP32 V-cycle, same workload, same timing ----
    timed_sol = S.get_sol_compact() if not args.no_compare else None
    solvers = None if args.no_compare else compare_solvers(S, prob, one, warm, torch, args, tuning)
    oracle = None if args.no_compare else oracle_check(S, prob, timed_sol)
    S.set_params(precision=args.precision, n_post_smooth=args.n_post, smoother=args.smoother,
                 inner_sweeps=args.inner_sweeps, learned=0, tol_rel=TOL, relax_omega=args.omega)
    S.prepare()

    # ---- roofline of the dominant kernel, timed live on the solver stream ----
    roof = roofline(S, prob, ext, torch, finest, args.precision, args.smoother)

    out = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 outer BiCGSTAB + %s V-cycle, f64 bottom" % ("f32" if args.precision == 1 else "f64"),
        "data": "synthetic",
        "config": {"workload": "%s: %s" % (args.config, WORKLOADS.get(args.config, "")) +
                               " (%dD, %d^%d-cell blocks, %d levels, %d leaf blocks)"
                               % (prob.ndim, prob.nb, prob.ndim, finest, len(prob.leaf)),
                   "leaf_cells": prob.leaf_cells, "blocks": prob.num_blocks, "tol_rel": TOL,
                   "l2": "flushed (256 MiB write) before every timed solve", "precision": args.precision,
                   "setting_tuning_ms": tuning,
                   "relax_omega": args.omega, "omega_tuning_ms": omega_tuning,
                   "iterations_per_solve": statistics.mean(iters), "n_post_smooth": args.n_post,
                   "smoother": ("red-black sweeps", "block-hybrid passes (Gauss-Seidel inside a block, Jacobi "
                                "between blocks), %d sweeps per pass" % args.inner_sweeps)[args.smoother],
                   "vcycle_kernel": ("per-phase launches", "cooperative", "cluster")[args.vcycle_kernel],
                   "cluster_cells": args.cluster_cells if args.vcycle_kernel == 2 else None,
                   "pdl": bool(args.pdl),
                   "sublevel_order": ("finest to coarsest per sublevel", "one launch per colour and level parity")[
                       args.sublevel_order],
                   "bottom_level": S.bottom_level(),
                   "constant_coef_blocks": S.uniform_blocks(),
                   "smoother_autotune": dict(zip(("variant", "us_per_variant"), S.tuned_smoother(args.precision))),
                   "parallelism": "replicas" if ws > 1 else "1 GPU"},
        "e2e": {"value": ws * prob.leaf_cells / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": clk.summary(),
        "solvers": solvers,
        "error_vs_oracle": oracle,
    }
    parts = getattr(prob, "parts", None)
    if rank == 0 and not args.no_cpu and parts:
        cs = cpu_batch_sample([cpu_payload(p) for p in parts])
        out["cpu_baseline"] = {"value": cs["value"], "unit": "cells/s", "cores": 1, "kind": "port",
                               "sample": ("the batch's first %d problems (%d leaf cells) each solved whole to 1e-8 "
                                          "by the C oracle (bit-exact restatement of the reference solver, bottom "
                                          "BiCGSTAB to 1e-10) on one host thread: %.1f s, %s outer iterations"
                                          % (cs["problems"], cs["cells"], cs["seconds"], cs["iterations"]))}
    elif rank == 0 and not args.no_cpu:
        big = prob.leaf_cells > CPU_FULL_CELLS
        cs = cpu_solve(prob, budget_s=CPU_SAMPLE_S if big else None,
                       n_iters=int(math.ceil(statistics.mean(iters))))
        if big:
            sample = ("%d outer iterations of this workload by the C oracle (bit-exact restatement of the "
                      "reference solver, bottom BiCGSTAB to 1e-10) on one host thread, %.2f s each, times the "
                      "%d iterations the device solve takes to 1e-8"
                      % (cs["sample_iterations"], cs["per_iteration"], cs["iterations"]))
        else:
            sample = ("one full solve of this workload to 1e-8 by the C oracle (bit-exact restatement of the "
                      "reference solver, bottom BiCGSTAB to 1e-10) on one host thread: %d outer iterations, "
                      "%.2f s" % (cs["iterations"], cs["seconds"]))
        out["cpu_baseline"] = {"value": cs["value"], "unit": "cells/s", "cores": 1, "kind": "port",
                               "sample": sample}
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()


# ---- config5 as a sequence: the elbow pipe with a moving sphere ----------
def _elbow_geometry(torch, tb, sc, seed):
    """the step's level set on every block's grown box (1 ghost layer, the
    reference's TreeData layout) and its right-hand side on every block's
    cells, computed with torch on the GPU and left there (the solver reads
    them in place): fluid = inside the tube and outside the sphere; rhs =
    -(8 seeded Gaussians, sigma 0.08) on the leaf blocks"""
    from sayakaamr_gb300 import workloads as W
    dev = "cuda"
    n, nb = tb["num_blocks"], tb["nb"]
    lo = torch.as_tensor(tb["block_lo"].reshape(n, 3), device=dev)
    dx = torch.as_tensor(tb["block_len"].reshape(n, 3) / nb, device=dev)

    def centres(G, shift):
        r = torch.arange(G, device=dev, dtype=torch.float64) + shift
        k, j, i = torch.meshgrid(r, r, r, indexing="ij")
        idx = torch.stack([i.reshape(-1), j.reshape(-1), k.reshape(-1)], 1)
        return lo[:, None, :] + idx[None] * dx[:, None, :]

    c = torch.as_tensor(W.ELBOW_C, device=dev)
    R = W.ELBOW_R

    def seg(p, a, b):
        a = torch.as_tensor(a, device=dev)
        b = torch.as_tensor(b, device=dev)
        ab = b - a
        t = torch.clamp(((p - a) * ab).sum(-1) / (ab * ab).sum(), 0.0, 1.0)
        return torch.linalg.norm(p - (a + t[..., None] * ab), dim=-1)

    def level_set(p):
        x, y, z = p[..., 0] - c[0], p[..., 1] - c[1], p[..., 2] - c[2]
        ang = torch.atan2(y, x)
        arc = torch.sqrt((torch.hypot(x, y) - R) ** 2 + z * z)
        d = torch.where((ang >= 0) & (ang <= 0.5 * math.pi), arc, torch.full_like(arc, float("inf")))
        d = torch.minimum(d, seg(p, [W.ELBOW_C[0] + R, 0.0, W.ELBOW_C[2]], [W.ELBOW_C[0] + R, W.ELBOW_C[1],
                                                                            W.ELBOW_C[2]]))
        d = torch.minimum(d, seg(p, [W.ELBOW_C[0], W.ELBOW_C[1] + R, W.ELBOW_C[2]], [0.0, W.ELBOW_C[1] + R,
                                                                                    W.ELBOW_C[2]]))
        sp = torch.linalg.norm(p - torch.as_tensor(sc, device=dev), dim=-1) - W.SPHERE_R
        return torch.minimum(W.ELBOW_TUBE - d, sp)

    ls = level_set(centres(nb + 2, -0.5)).reshape(-1).contiguous()
    pc = centres(nb, 0.5)
    g = torch.Generator(device="cpu").manual_seed(seed)
    amp = torch.randn(8, generator=g, dtype=torch.float64).to(dev)
    cen = (0.1 + 0.8 * torch.rand(8, 3, generator=g, dtype=torch.float64)).to(dev)
    f = torch.zeros(pc.shape[:2], dtype=torch.float64, device=dev)
    for q in range(8):
        f += amp[q] * torch.exp(-((pc - cen[q]) ** 2).sum(-1) / (2 * 0.08 ** 2))
    leaf = torch.as_tensor(tb["node_type"] == 1, device=dev)
    rhs = (-f * leaf[:, None]).reshape(-1).contiguous()
    return ls, rhs


def run_sequence(args, torch, ws, rank, local):
    """--sequence K (config5): K pressure solves of the elbow while the
    sphere moves from 10% to 90% of the centreline; every --regrid-every
    steps the tree is regridded toward the sphere's new position (host tree
    mirror) and a new solver is built on it, warm-started from the old
    solution by the device regrid transfer; between regrids the solver takes
    the step's fractions (setIBFracByLS from the level set, on the device)
    and right-hand side and solves from the previous solution.  Timed per
    step (wall clock, host synchronised): the solver's setup (tree upload,
    coefficients, prepare) and the solve; the geometry (level set and
    right-hand side, computed with torch) and the host tree regrid are
    reported beside it, outside the solver time."""
    import sayakaamr_gb300 as sg
    from sayakaamr_gb300 import workloads as W
    if args.config != "config5":
        raise SystemExit("--sequence runs the config5 elbow sequence")
    K, every = args.sequence, max(1, args.regrid_every)
    # the dense bottom solve on level 1 (512 cells per component here): its
    # inverse is rebuilt in milliseconds after a regrid, where level 2's
    # (4096 cells) takes about 0.26 s
    prm = dict(tol_rel=TOL, tol_abs=0.0, use_mg_precond=1, max_iter=2000, bottom=1, graph=1,
               precision=1 if args.precision < 0 else args.precision,
               n_post_smooth=4 if args.n_post < 0 else args.n_post,
               bottom_level=args.bottom_level if args.bottom_level > 0 else 1,
               bottom_refresh=args.bottom_refresh, smoother=max(args.smoother, 0),
               # over-relaxed sweeps: 3.4 instead of 4.0 iterations per solve
               # on the 100-solve elbow sequence (29.8 vs 33.3 ms per step)
               relax_omega=args.omega if args.omega > 0 else 1.1)
    t0 = time.perf_counter()
    sc = W.elbow_point(0.1)
    tree = W.elbow_tree(sc, max_level=args.max_level)
    tree_build_s = time.perf_counter() - t0
    S = None
    steps = []
    geo_s = regrid_tree_s = 0.0
    cells = 0
    for k in range(K):
        sc = W.elbow_point(0.1 + 0.8 * k / max(1, K - 1))
        new_tree = k == 0 or k % every == 0
        if k > 0 and new_tree:
            t0 = time.perf_counter()
            W.elbow_regrid(tree, sc, args.max_level)
            regrid_tree_s += time.perf_counter() - t0
        if new_tree:
            tb = tree.tables()
            n = tb["num_blocks"]
            bc = np.full((n, 6), -1, dtype=np.int32)
            nbr = tb["neighbor"].reshape(n, 6)
            for fc in range(6):
                bc[nbr[:, fc] <= -20, fc] = sg.DIRICHLET if fc == 0 else sg.NEUMANN
            leaf_cells = int((tb["node_type"] == 1).sum()) * tb["nb"] ** 3
        t0 = time.perf_counter()
        ls, rhs = _elbow_geometry(torch, tb, sc, 5000 + k)
        geo_s += time.perf_counter() - t0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ph = {}

        def mark(name, t_prev, solver):
            torch.cuda.ExternalStream(solver.stream()).synchronize()
            now = time.perf_counter()
            ph[name] = (now - t_prev) * 1e3
            return now
        if new_tree:
            S2 = sg.MacSolver(tb)
            S2.set_bc(bc.reshape(-1))
            ta = mark("create", t0, S2)
            S2.set_ib_frac_by_ls_device(ls.data_ptr(), ngrow=1)
            ta = mark("fractions", ta, S2)
            S2.set_params(**prm)
            if S is None:
                S2.set_zero_sol()
            else:
                S2.init_from(S, prolong=args.transfer)
            ta = mark("transfer", ta, S2)
            S = S2
        else:
            S.set_ib_frac_by_ls_device(ls.data_ptr(), ngrow=1)
            ta = mark("fractions", t0, S)
        S.set_rhs_device(rhs.data_ptr())
        ta = mark("rhs", ta, S)
        S.prepare()
        mark("prepare", ta, S)
        t1 = time.perf_counter()
        if k == 0 and prm.get("smooth_variant", -1) < 0:
            # later trees of the sequence use the variant the first one tuned
            prm["smooth_variant"] = S.tuned_smoother(prm["precision"])[0]
        S.cg_solve_async()
        info = S.solve_info()
        t2 = time.perf_counter()
        if info["status"] != 0 or not info["rnorm"] < TOL * info["rnorm0"]:
            raise SystemExit("sequence step %d did not converge: %s" % (k, info))
        steps.append(dict(setup_s=t1 - t0, solve_s=t2 - t1, iterations=info["iterations"], new_tree=new_tree,
                          blocks=int(tb["num_blocks"]), leaf_cells=leaf_cells, phases=ph))
        cells += leaf_cells
    total = sum(r["setup_s"] + r["solve_s"] for r in steps)
    setup = sum(r["setup_s"] for r in steps)
    its = [r["iterations"] for r in steps]
    out = {
        "metric": METRIC, "value": cells / total, "unit": "cells/s", "n_gpus": ws, "steps": K, "warmup": 0,
        "ms_per_step": total / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 outer BiCGSTAB + %s V-cycle, f64 bottom" % ("f32" if prm["precision"] == 1 else "f64"),
        "data": "synthetic",
        "config": {"workload": "config5 sequence: elbow pipe (tube 0.1, bend 0.3), sphere r=0.04 moving from 10%% "
                               "to 90%% of the centreline over %d solves, regrid every %d, %d^3-cell blocks, up to "
                               "%d levels, binary IB from the level set (setIBFracByLS), p=0 outlet"
                               % (K, every, 8, args.max_level),
                   "tol_rel": TOL, "params": prm, "transfer": args.transfer},
        "sequence": {"total_s": total, "setup_s": setup, "setup_share": setup / total,
                     "solve_s": total - setup, "regrids": sum(1 for r in steps if r["new_tree"]) - 1,
                     "iterations_mean": statistics.mean(its), "iterations_max": max(its),
                     "setup_s_regrid_steps": sum(r["setup_s"] for r in steps if r["new_tree"]),
                     "setup_s_other_steps": sum(r["setup_s"] for r in steps if not r["new_tree"]),
                     "geometry_s_outside": geo_s, "host_tree_regrid_s_outside": regrid_tree_s,
                     "initial_tree_s_outside": tree_build_s,
                     "per_step": [[round(r["setup_s"] * 1e3, 2), round(r["solve_s"] * 1e3, 2), r["iterations"]]
                                  for r in steps],
                     "per_step_columns": ["setup ms", "solve ms", "iterations"],
                     "setup_phases_ms_regrid_step": steps[every if K > every else 0]["phases"],
                     "setup_phases_ms_other_step": steps[1 if K > 1 else 0]["phases"]},
    }
    if rank == 0:
        print(json.dumps(out))


def compare_solvers(S, prob, one, warm, torch, args, tuning):
    """time to 1e-8 (ms, CUDA events, L2 flushed) and iterations of: plain
    FP64 MG-BiCGSTAB (FP64 V-cycle, the reference's 2 post-smoothing sweeps),
    the FP32 V-cycle with the tuned sweeps, and the learned block correction
    with the FP32 V-cycle (trained on this workload's own solver iterates
    first, 2D only)"""
    fp32 = dict(precision=1, n_post_smooth=args.n_post, smoother=args.smoother, inner_sweeps=args.inner_sweeps,
                relax_omega=args.omega)
    if tuning:
        t32 = [r for r in tuning if r["precision"] == 1 and r["ms"] is not None]
        if t32:
            b = min(t32, key=lambda r: r["ms"])
            fp32 = dict(precision=1, n_post_smooth=b["n_post_smooth"], smoother=b["smoother"],
                        inner_sweeps=b["inner_sweeps"], relax_omega=args.omega)
    # the reference's method on the device: FP64 V-cycle, red-black
    # Gauss-Seidel with its default 2 post-smoothing sweeps
    settings = [("plain_fp64_mg", dict(precision=0, n_post_smooth=2, smoother=0, inner_sweeps=2, learned=0,
                                       relax_omega=1.0)),
                ("fp32_vcycle", dict(fp32, learned=0))]
    out = {}
    learned_note = None
    if prob.ndim == 2 and prob.nb in (8, 16):
        S.set_params(**dict(fp32, learned=0))
        t0 = time.perf_counter()
        info = S.learned_train_on_workload()
        learned_note = dict(train_seconds=time.perf_counter() - t0, **info)
        settings.append(("learned_fp32_vcycle", dict(fp32, learned=1)))
    for label, prm in settings:
        S.set_params(**prm)
        S.prepare()
        try:
            # status 3: converged after the learned correction was switched off
            warm(dict(label=label, **prm), ok=(0, 3))
        except SystemExit as e:
            out[label] = {"failed": str(e)}
            continue
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
        infos = [one(e) for e in ev]
        torch.cuda.synchronize()
        if any(i["status"] not in (0, 3) for i in infos):
            out[label] = {"failed": infos[0]}
            continue
        out[label] = {"ms": statistics.mean(a.elapsed_time(b) for a, b in ev),
                      "iterations": statistics.mean(i["iterations"] for i in infos),
                      "setting": {k: v for k, v in prm.items() if k != "learned"},
                      "stall_fallback": any(i["status"] == 3 for i in infos)}
    if learned_note:
        out["learned_training"] = learned_note
    S.set_params(learned=0)
    return out


def kernel_only(S, prob, ext, torch, args):
    """args.warmup + args.steps launches of one kernel on the solver stream"""
    finest = int(prob.tables["level"].max())
    for _ in range(args.warmup):
        S.enqueue_kernel(args.kernel, finest)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(ext)
    for _ in range(args.steps):
        S.enqueue_kernel(args.kernel, finest)
    b.record(ext)
    torch.cuda.synchronize()
    cells = S.tower_size(finest, finest) * prob.ncell
    print(json.dumps({"kernel": args.kernel, "config": args.config, "launches": args.steps,
                      "us_per_launch": a.elapsed_time(b) * 1e3 / args.steps, "cells_of_the_level": cells}))


# ncu summaries of the dominant sweep per (workload, V-cycle precision)
PROFILES = {("config2", 0): "k_rbgs_config2.md", ("config2", 1): "k_rbgs_f32_config2.md",
            ("config3", 1): "k_rbgs_tile_config3.md", ("config4", 1): "k_rbgs_warp16_config4.md"}


def profiled_traffic(workload, precision):
    """DRAM bytes per launch (read + write) from the committed ncu summary of
    this workload's smoother sweep, or None"""
    import re
    name = PROFILES.get((workload, precision))
    if not name:
        return None, None
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None, None
    m = re.search(r"dram__bytes_read\.sum \+ dram__bytes_write\.sum \| .*= ([0-9.]+) MB", open(path).read())
    if not m:
        return None, None
    return float(m.group(1)) * 1e6, "profiles/" + name


def roofline(S, prob, ext, torch, finest, precision, smoother=0):
    """dominant kernel: the red-black sweep (one colour) over the finest level
    of the finest tower, in the V-cycle's precision, with the variant the
    autotuner chose.  Algorithmic bytes per launch = cells of that level x
    p x (2 + ndim) (p = 4 or 8 bytes): phi of the other colour read and the
    updated colour written (p/2 + p/2), rhs and vf of the updated colour
    (p/2 + p/2) and every face coefficient of the level (ndim x p)."""
    import json as _json
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(_json.load(f)["hbm_gbs"])
            src = "measured"
    which = 1 if precision == 1 else 2
    p = 4 if precision == 1 else 8
    nblk = S.tower_size(finest, finest)
    cells = nblk * prob.ncell
    bytes_per_launch = cells * p * (2 + prob.ndim)
    reps = 200
    for _ in range(10):
        S.enqueue_kernel(which, finest)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(ext)
    for _ in range(reps):
        S.enqueue_kernel(which, finest)
    b.record(ext)
    torch.cuda.synchronize()
    us = a.elapsed_time(b) * 1e3 / reps
    achieved = bytes_per_launch / (us * 1e-6) / 1e9
    variant, _ = S.tuned_smoother(precision)
    traffic, traffic_src = profiled_traffic(prob.name, precision)
    warp = variant in (11, 12) and prob.ndim == 2 and prob.nb == 16 and p == 4
    kind = ("k_rbgs (one thread per cell)" if variant <= 4 or (variant >= 11 and not warp) else
            "k_rbgs_tile (block staged in shared memory)" if variant <= 7 else
            "k_rbgs_bulk (tile and faces staged by TMA bulk copies)" if variant == 8 else
            "k_rbgs_stream (persistent, double-buffered bulk copies)" if variant == 9 else
            "k_rbgs_ilp (two cells per thread)" if variant == 10 else
            "k_rbgs_warp16 (one warp per block, registers and shuffles)")
    l2 = bytes_per_launch < 100e6
    return {"kernel": "%s<%s,%dD>, autotuned variant %d, finest level, one colour"
                      % (kind, "float" if p == 4 else "double", prob.ndim, variant),
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "traffic_source": traffic_src,
            "bytes_per_launch": bytes_per_launch, "us_per_launch": us,
            "peak_source": src + " (burst copy)",
            "note": ("working set fits in L2 at this size: latency-bound; " if l2 else "") +
                    ("the setting chosen smooths with block-hybrid passes (k_bhgs), which read the same "
                     "arrays once per pass; " if smoother == 1 else "") +
                    "DRAM traffic per launch from the ncu summaries"}


if __name__ == "__main__":
    main()
