"""Benchmark: SCF solves/s at |residual| < 1e-7 on a stream of batched brushes.

Workload (one "step"): 512 independent 1-gradient planar brushes solved to
‖g‖₂ < 1e-7, drawn from a fixed seed: n_layers ~ U{50..400}, N ~ U{20..500},
σ ~ U[0.01, 0.1], χ_AS ~ U[0, 1]; every 10th instance is a 3-arm star with
arms of N/3 joined at a branch point.  Every step solves them from a fresh
seeded start field u ~ U(-0.01, 0.01).  The K timed steps run through one
device-resident work loop (resident 128-thread CTAs taking problems from a
queue, DIIS on the device): FP32 block-floating-point propagators, FP64
normalisation, residual and DIIS, and an FP64-propagator finish in the same
CTA.  Beside it: the same stream with FP64 propagators throughout
(`fp64_gpu`), the plain FP64 GPU path that solves one problem at a time
through a device context (`fp64_gpu_unbatched`), and the p50/p99 of the
per-problem time to convergence (device timer).

Contract: `python bench.py --gpus N --steps K --warmup W` prints one JSON
line.  `value` times the kernel with inputs resident in HBM (CUDA events);
`e2e` times the C-ABI call with host buffers (nm_batch_solve_host: host→device
copy of the fields, solve, device→host copy of the solution).
`--impl reference` times the CPU restatement of the reference path
(oracle/scf_oracle.c, one solve per host thread) on a bounded sample.
Multi-GPU: the instances are independent solves, so N GPUs run N replicas of
the same workload with no collective (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
# more hardware work queues than streams: a stream that shares a queue with
# the persistent work loop's stream would wait behind the loop (read when
# the CUDA context is created, so set before torch or the library touch it)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

N_INSTANCES = 512
SEED = 20251203
FIELD = (-0.01, 0.01)
METRIC = "SCF solves/s at |residual|<1e-7 (served FP32 vs plain FP64 GPU); p50/p99 latency"
UNIT = "solves/s"
B_PER_UPDATE_FP32 = 22.0   # algorithmic bytes per segment-site update (FP32 propagators, FP64 φ)
B_PER_UPDATE_FP64 = 36.0


def instance_text(nl: int, N: int, sigma: float, chi: float, star: bool) -> str:
    if star:
        a = max(N // 3, 2)
        comp = f"(X)1(A){a - 1}[(A){a}](A){a}"
    else:
        comp = f"(X)1(A){N - 1}"
    return "\n".join([
        f"lat : flat : n_layers : {nl}", "lat : flat : lattice_type : simple_cubic",
        "lat : flat : geometry : planar", "lat : flat : gradients : 1",
        "lat : flat : lowerbound : surface", "lat : flat : upperbound : mirror",
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : X : freedom : pinned", "mon : X : pinned_range : firstlayer",
        "mon : A : freedom : free", "mon : W : freedom : free",
        f"mon : A : chi_W : {chi:.6f}", f"mon : X : chi_W : {chi:.6f}",
        f"mol : pol : composition : {comp}", "mol : pol : freedom : restricted",
        f"mol : pol : n : {sigma:.6f}",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent",
        "newton : isaac : method : DIIS", "newton : isaac : tolerance : 1e-7",
        "newton : isaac : deltamax : 0.1", "newton : isaac : iterationlimit : 1000",
    ]) + "\n"


def workload(n: int = N_INSTANCES):
    """Seeded instances.  Draws whose grafted amount θ = σN exceeds 40% of
    the lattice (a brush that would fill the box; the reference itself
    refuses θ > volume, molecule.cpp CheckInput) are redrawn."""
    rng = np.random.default_rng(SEED)
    out = []
    for i in range(n):
        while True:
            nl = int(rng.integers(50, 401))
            N = int(rng.integers(20, 501))
            sigma = float(rng.uniform(0.01, 0.1))
            chi = float(rng.uniform(0.0, 1.0))
            if sigma * N <= 0.4 * nl:
                break
        out.append(instance_text(nl, N, sigma, chi, star=(i % 10 == 9)))
    return out


def fields(plans, seed=SEED + 1):
    rng = np.random.default_rng(seed)
    return [rng.uniform(*FIELD, size=p.iv) for p in plans]


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_over_ranks(ms: float, e2e_s: float, n_ok: int, device="cuda"):
    """Whole-job figures of N replicas: the slowest rank's step time and
    end-to-end time (max over ranks) and the converged solves of all ranks
    (sum).  Without a process group, or with one rank, the figures as given."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms, e2e_s, n_ok
    t = torch.tensor([ms, e2e_s], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([n_ok], dtype=torch.int64, device=device)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t[0]), float(t[1]), int(n[0])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        try:
            for ln in self.path.read_text().splitlines():
                t = [s.strip() for s in ln.split(",")]
                if len(t) < 9:
                    continue
                try:
                    sm.append(float(t[1]))
                    mx = float(t[2])
                except ValueError:
                    continue
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                for nm, v in zip(names, t[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except Exception:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _oracle_pool(plans, xs, threads: int, budget_s: float | None = None):
    """The oracle's DIIS solve of each problem (oracle/scf_oracle.c, the CPU
    restatement of the reference path), one solve at a time per host thread
    (the reference's Solve is single-threaded), until every problem is done
    or budget_s has passed.  Returns (attempted, converged, seconds)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from orc import Oracle
    lock = threading.Lock()
    state = {"next": 0, "done": 0, "ok": 0}
    t0 = time.perf_counter()

    def worker():
        while True:
            with lock:
                i = state["next"]
                if i >= len(plans) or (budget_s is not None and time.perf_counter() - t0 > budget_s):
                    return
                state["next"] += 1
            rc, _, its, res = Oracle(plans[i]).solve(xs[i])
            with lock:
                state["done"] += 1
                state["ok"] += rc == 0 and res <= plans[i].rec.tolerance  # converged solves only
    ts = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return state["done"], state["ok"], time.perf_counter() - t0


def cpu_baseline(texts, xs, budget_s: float = 15.0, threads: int | None = None) -> dict:
    """The CPU restatement of the reference path on all host threads over the
    instances of one step (problems built by the oracle's own plan builder;
    the product library is not used)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from orc_plan import OraclePlan
    threads = threads or os.cpu_count() or 1
    plans = [OraclePlan(t) for t in texts]
    done, ok, dt = _oracle_pool(plans, xs, threads, budget_s)
    return {"value": ok / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {done} of {len(texts)} instances of one step ({ok} converged), one solve per "
                      f"thread, {dt:.1f} s wall",
            "seconds": dt}


def run_reference(args) -> None:
    """The reference arm: the CPU restatement of the reference's solve on the
    host cores, over the SAME steps as the device arm: every step the 512
    instances from that step's seeded fields (step k: seed SEED + 1 + k), one
    solve per host thread at a time.  Problems are built by the oracle's own
    plan builder (oracle/orc_plan.py); only oracle/liborc.so is loaded.  The
    reference program itself is built from its sources only where they are
    (x86 here); its binary does not run on the Arm host of the GPU."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from namics_gb300 import build as b  # the build recipe only; no library is loaded
    b.build_oracle()
    sys.path.insert(0, str(ROOT / "oracle"))
    from orc_plan import OraclePlan
    texts = workload(args.instances)
    plans = [OraclePlan(t) for t in texts]
    threads = os.cpu_count() or 1
    for k in range(args.warmup):
        _oracle_pool(plans, fields(plans, seed=SEED + 1001 + k), threads)
    tot_ok, tot_s, tot = 0, 0.0, 0
    for k in range(args.steps):
        done, ok, dt = _oracle_pool(plans, fields(plans, seed=SEED + 1 + k), threads)
        tot_ok += ok
        tot_s += dt
        tot += done
    v = tot_ok / tot_s
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_s / args.steps * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": "stream of batched 1-gradient brushes/stars: 512 seeded instances per step, "
                                   "each step from fresh seeded fields (the device arm's steps)",
                       "instances_per_step": len(texts), "solves": tot, "converged": tot_ok},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"all {len(texts)} instances of each of {args.steps} steps, one solve per "
                                       "host thread at a time"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def melt3d_text(n: int = 128, itlim: int = 20) -> str:
    """The 3-D melt: n³ box, periodic in all three directions, melt of symmetric
    diblock (A)50(B)50 (N = 100, incompressible), chi_AB = 0.3."""
    return "\n".join([
        "lat : flat : gradients : 3", f"lat : flat : n_layers_x : {n}", f"lat : flat : n_layers_y : {n}",
        f"lat : flat : n_layers_z : {n}", "lat : flat : geometry : planar", "lat : flat : lattice_type : simple_cubic",
    ] + [f"lat : flat : {b}bound_{a} : periodic" for a in "xyz" for b in ("lower", "upper")] + [
        "mon : A : freedom : free", "mon : B : freedom : free", "mon : A : chi_B : 0.3",
        "mol : AB : composition : (A)50(B)50", "mol : AB : freedom : solvent",
        "newton : isaac : method : DIIS", "newton : isaac : tolerance : 1e-7",
        f"newton : isaac : iterationlimit : {itlim}", "newton : isaac : deltamax : 0.1", "newton : isaac : m : 10",
    ]) + "\n"


def run_melt3d(args) -> dict:
    """On one GPU: DIIS iterations of the 128³ A50B50 melt with FP32
    propagators (per-vector power-of-two exponents, FP64 DIIS) and with plain
    FP64 propagators, from the same seeded field u_A = -u_B ~ U(-0.1, 0.1).
    A step is `--iters` DIIS iterations (residual + field update), timed with
    CUDA events on the context's stream; L2 is flushed between steps (the
    propagators, 1.76 GB in FP64, exceed L2 anyway).  The reference's DIIS does
    not reach |g| < 1e-7 on this input (deltamax 0.1 ends in NaN after ~60
    iterations on a 32³ box in the CPU restatement; 0.01 leaves |g| = 0.1
    after 3000), so the metric is iterations/s, not solves/s."""
    import torch
    from namics_gb300 import build as b
    b.build_product()
    from namics_gb300 import NM_FP32, NM_FP64, Context, Plan
    n = args.n3d
    plan = Plan(melt3d_text(n, args.iters))
    rng = np.random.default_rng(SEED)
    u = rng.uniform(-0.1, 0.1, size=plan.M)
    x0 = torch.from_numpy(np.concatenate([u, -u])).cuda()
    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    out = {}
    arms = ((NM_FP32, "fp32", args.ckpt), (NM_FP32, "fp32_full_storage", 0), (NM_FP32, "fp32_autotuned", -1),
            (NM_FP64, "fp64", 0))
    for prec, name, ck in arms:
        ctx = Context(plan, prec, stream=stream.cuda_stream, checkpoint_stride=max(ck, 0))
        tuned = ctx.autotune(x0.data_ptr()) if ck < 0 else None
        xw = torch.empty_like(x0)
        times = []
        for k in range(args.warmup + args.steps):
            flush.zero_()
            xw.copy_(x0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = ctx.solve_dev(xw.data_ptr())
            e1.record(stream)
            e1.synchronize()
            if k >= args.warmup:
                times.append(e0.elapsed_time(e1))
        ms = statistics.mean(times)
        its = r.iterations + 1  # residual evaluations: the first plus one per iteration
        out[name] = {"ms_per_step": ms, "residuals_per_step": its, "ms_per_residual_and_update": ms / its,
                     "launches": ctx.launch_count(), "checkpoint_stride": ck}
        if tuned:
            out[name].update(autotuned=tuned, checkpoint_stride=tuned["checkpoint_stride"])
        ctx.close()
    updates = 2.0 * 100 * n ** 3  # segment-site updates per residual
    f32, f64 = out["fp32"], out["fp64"]
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = B_PER_UPDATE_FP32 * updates / (f32["ms_per_residual_and_update"] / 1000.0) / 1e9
    line = {
        "metric": "SCF DIIS iterations/s, 128^3 A50B50 melt (FP32 propagators vs plain FP64 GPU)",
        "value": 1000.0 / f32["ms_per_residual_and_update"], "unit": "iterations/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": f32["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded field)",
        "config": {"workload": f"{n}^3 periodic (A)50(B)50 melt, chi_AB 0.3, u_A=-u_B~U(-0.1,0.1), "
                               f"propagators checkpointed every {args.ckpt} segments",
                   "iterations_per_step": args.iters, "l2": "flushed between steps (256 MB write)",
                   "segment_site_updates_per_residual": updates, "parallelism": "one GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None,
                     "note": "22 B per segment-site update x updates / (residual + DIIS update) time; peak of "
                             "measured (MEASURED_PEAKS.json hbm_gbs)"},
        "updates_per_s": updates / (f32["ms_per_residual_and_update"] / 1000.0),
        "fp32": f32, "fp32_full_storage": out["fp32_full_storage"], "fp32_autotuned": out["fp32_autotuned"],
        "fp64_gpu": dict(f64, value=1000.0 / f64["ms_per_residual_and_update"], unit="iterations/s"),
    }
    return line


def ads2d_text(n: int = 100, N: int = 200) -> str:
    """Request stream, 25% of requests: 2-D planar n×n adsorption of (A)N from a
    bulk at phi_b = 1e-3 onto a surface with chi_AS = -1, monomeric solvent."""
    return "\n".join([
        "lat : flat : gradients : 2", f"lat : flat : n_layers_x : {n}", f"lat : flat : n_layers_y : {n}",
        "lat : flat : geometry : planar", "lat : flat : lattice_type : simple_cubic",
        "lat : flat : lowerbound_x : surface", "lat : flat : upperbound_x : mirror",
        "lat : flat : lowerbound_y : mirror", "lat : flat : upperbound_y : mirror",
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : A : freedom : free", "mon : W : freedom : free", "mon : A : chi_S : -1",
        f"mol : pol : composition : (A){N}", "mol : pol : freedom : free", "mol : pol : phibulk : 1e-3",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent",
        "newton : isaac : method : DIIS", "newton : isaac : tolerance : 1e-7",
        "newton : isaac : iterationlimit : 1000", "newton : isaac : deltamax : 0.1", "newton : isaac : m : 10",
    ]) + "\n"


def melt3d_small_text(n: int = 64, a: int = 20, chi: float = 0.4) -> str:
    """Request stream, 5% of requests: n³ periodic (A)a(B)a melt at chi_AB."""
    return melt3d_text(n, 1000).replace("chi_B : 0.3", f"chi_B : {chi}").replace(
        "(A)50(B)50", f"(A){a}(B){a}")


def cyl2d_text(nx: int = 200, ny: int = 200, N: int = 500, n: float = 1.0, chi: float = 0.5,
               itlim: int = 20, tol: float = 1e-7) -> str:
    """The charged cylindrical brush: 2-D cylindrical nx (r) × ny (z) lattice, offset_first_layer
    10 (inner cylinder of radius 10, a frozen wall below x = 1), (X)1(A)N-1
    pinned at the first layer with n chains, chi_AS = chi; A carries valence
    -0.1, monovalent ions: Na the neutraliser, Cl free at phi_b 0.01; water
    the solvent; bondlength 5e-10 m."""
    return "\n".join([
        "lat : flat : gradients : 2", f"lat : flat : n_layers_x : {nx}", f"lat : flat : n_layers_y : {ny}",
        "lat : flat : geometry : cylindrical", "lat : flat : lattice_type : simple_cubic",
        "lat : flat : offset_first_layer : 10", "lat : flat : bondlength : 5e-10",
        "lat : flat : lowerbound_x : surface", "lat : flat : upperbound_x : mirror",
        "lat : flat : lowerbound_y : mirror", "lat : flat : upperbound_y : mirror",
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : X : freedom : pinned", "mon : X : pinned_range : firstlayer",
        "mon : A : freedom : free", "mon : A : valence : -0.1", "mon : W : freedom : free",
        "mon : Na : freedom : free", "mon : Na : valence : 1", "mon : Cl : freedom : free", "mon : Cl : valence : -1",
        f"mon : A : chi_W : {chi}", f"mon : X : chi_W : {chi}",
        f"mol : pol : composition : (X)1(A){N - 1}", "mol : pol : freedom : restricted", f"mol : pol : n : {n!r}",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent",
        "mol : Na : composition : (Na)1", "mol : Na : freedom : neutralizer",
        "mol : Cl : composition : (Cl)1", "mol : Cl : freedom : free", "mol : Cl : phibulk : 0.01",
        "newton : isaac : method : DIIS", f"newton : isaac : tolerance : {tol}",
        f"newton : isaac : iterationlimit : {itlim}", "newton : isaac : deltamax : 0.1", "newton : isaac : m : 10",
    ]) + "\n"


def cyl2d_plan(nx: int, ny: int, N: int, sigma: float, chi: float, itlim: int, tol: float = 1e-7):
    """The charged cylindrical brush with n = sigma × (sites of the first layer, Σ_y L(x=1))."""
    from namics_gb300 import Plan
    probe = Plan(cyl2d_text(nx, ny, N, 1.0, chi, itlim, tol))
    c = probe.c
    first = sum(c.L[1 * c.JX + y] for y in range(1, ny + 1))
    return Plan(cyl2d_text(nx, ny, N, sigma * first, chi, itlim, tol))


def run_cyl2d(args) -> dict:
    """On one GPU: the 200×200 cylindrical charged brush (A_500, sigma
    0.02, A valence -0.1, Na neutraliser, Cl phi_b 0.01) at both chi_AS values
    of the configuration, 0 and 0.5, solved side by side: one device context
    and one CUDA stream each, driven from two host threads.  A single solve
    is latency-bound (40 804 sites per step), so the two overlap on the GPU.
    Start fields x ~ U(-0.01, 0.01), ψ included, seeded.

    A step is `--iters` DIIS iterations (residual + Poisson update + field
    update) of both solves; its time is the larger of the two streams' CUDA
    event intervals, both started after a device synchronisation; L2 is
    flushed between steps.  `value` = DIIS iterations of both solves per
    second.  Arms: FP32 propagators (one power-of-two exponent per lattice
    row; FP64 composition, Poisson update, residual and DIIS) and plain FP64.
    Also per arm: the max |Δφ| of one residual at the seeded field against the
    CPU oracle, and both full solves to ‖g‖ < 1e-7 side by side (FP32 arm:
    FP32 first, FP64 finish), timed end to end."""
    import torch
    from namics_gb300 import build as b
    b.build_product()
    from namics_gb300 import NM_FP32, NM_FP64, Context
    nx = ny = args.n2d
    chis = (0.0, 0.5)
    plans = [cyl2d_plan(nx, ny, 500, 0.02, c, args.iters) for c in chis]
    solve_plans = [cyl2d_plan(nx, ny, 500, 0.02, c, 20000) for c in chis]
    # one seeded field per plan: the iteration vector's length depends on chi
    # (at chi_AS = 0 every segment shares one chi row, one iteration species)
    x0h = [np.random.default_rng(SEED + i).uniform(-0.01, 0.01, size=p.iv) for i, p in enumerate(plans)]
    for p, sp, xh in zip(plans, solve_plans, x0h):
        assert p.iv == sp.iv == xh.size
    x0 = [torch.from_numpy(xh).cuda() for xh in x0h]
    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device="cuda")
    streams = [torch.cuda.Stream() for _ in chis]

    def side_by_side(fns):
        th = [threading.Thread(target=f) for f in fns]
        for t in th:
            t.start()
        for t in th:
            t.join()

    out = {}
    for prec, name in ((NM_FP32, "fp32"), (NM_FP64, "fp64")):
        ctxs = [Context(p, prec, stream=st.cuda_stream) for p, st in zip(plans, streams)]
        xw = [torch.empty_like(x) for x in x0]
        times, its = [], []
        res = [None, None]
        clocks = ClockSampler(0)
        with clocks:
            for k in range(args.warmup + args.steps):
                flush.zero_()
                for w, x in zip(xw, x0):
                    w.copy_(x)
                torch.cuda.synchronize()
                ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in chis]
                for (e0, _), st in zip(ev, streams):
                    e0.record(st)

                def run(i):
                    res[i] = ctxs[i].solve_dev(xw[i].data_ptr())
                    ev[i][1].record(streams[i])

                side_by_side([lambda i=i: run(i) for i in range(len(chis))])
                for _, e1 in ev:
                    e1.synchronize()
                if k >= args.warmup:
                    times.append(max(e0.elapsed_time(e1) for e0, e1 in ev))
                    its.append(sum(r.iterations + 1 for r in res))
        ms = statistics.mean(times)
        n_its = statistics.mean(its)
        out[name] = {"ms_per_step": ms, "residuals_per_step": n_its, "iterations_per_s": 1000.0 * n_its / ms,
                     "residual_after_step": [r.residual for r in res],
                     "launches": sum(c.launch_count() for c in ctxs), "clocks": clocks.summary()}
        gd = torch.zeros_like(x0[1])
        ctxs[1].residual_dev(x0[1].data_ptr(), gd.data_ptr())
        out[name]["phi"] = ctxs[1].field(0)
        for c in ctxs:
            c.close()
        if not args.no_solve:
            sctx = [Context(p, prec, stream=st.cuda_stream) for p, st in zip(solve_plans, streams)]
            xs = [xh.copy() for xh in x0h]
            rs = [None, None]

            def solve(i):
                rs[i], _ = sctx[i].solve_host(xs[i], want_phi=False)

            t0 = time.perf_counter()
            side_by_side([lambda i=i: solve(i) for i in range(len(chis))])
            out[name]["full_solves"] = {"seconds_both": time.perf_counter() - t0,
                                        "iterations": [r.iterations for r in rs],
                                        "residual": [r.residual for r in rs], "status": [r.status for r in rs]}
            for c in sctx:
                c.close()
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        b.build_oracle()
        from orc import Oracle
        orc = Oracle(plans[1])
        rc, _ = orc.residual(x0h[1])
        if rc == 0:
            mask = np.tile(plans[1].interior_mask(), plans[1].n_seg)
            po = orc.field(0)[mask]
            for name in out:
                out[name]["max_abs_dphi_vs_oracle"] = float(np.max(np.abs(out[name]["phi"][mask] - po)))
    f32, f64 = out["fp32"], out["fp64"]
    updates = float(plans[0].segment_updates())
    line = {
        "metric": "SCF DIIS iterations/s, 200x200 cylindrical charged brush A500 at chi_AS 0 and 0.5 side by side "
                  "(FP32 propagators vs plain FP64 GPU)",
        "value": f32["iterations_per_s"], "unit": "iterations/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": f32["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded field)",
        "config": {"workload": f"{nx}x{ny} cylindrical charged brush, offset 10, (X)1(A)499 pinned, sigma 0.02, "
                               "chi_AS in {0, 0.5} (two solves side by side), A valence -0.1, Na neutraliser, "
                               "Cl phi_b 0.01, bondlength 5e-10",
                   "iterations_per_step": args.iters, "l2": "flushed between steps (256 MB write)",
                   "segment_site_updates_per_residual": updates, "parallelism": "one GPU, two streams"},
        "updates_per_s": updates * f32["iterations_per_s"],
        "fp32": {k: v for k, v in f32.items() if k != "phi"},
        "fp64_gpu": dict({k: v for k, v in f64.items() if k != "phi"},
                         value=f64["iterations_per_s"], unit="iterations/s"),
    }
    return line


def weak2d_text(nx: int = 100, ny: int = 100, N: int = 200, n: float = 1.0, h3o: str = "1e-7",
                itlim: int = 20, tol: float = 1e-7) -> str:
    """A weak-polyacid brush with internal states on a 2-D planar nx × ny
    lattice: (X)1(A)N-1 pinned at the first layer (n chains), a frozen wall
    below; A has states AH (neutral, χ 0.8 with H2O) and AM (charge -1),
    water states H3O+ (bulk fraction h3o), H2O and OH-; reactions AH + H2O =
    AM + H3O+ (pK 6) and 2 H2O = OH- + H3O+ (pK 14); Na neutraliser, Cl at
    φ_b 0.01; bondlength 3e-10."""
    return "\n".join([
        "lat : flat : gradients : 2", f"lat : flat : n_layers_x : {nx}", f"lat : flat : n_layers_y : {ny}",
        "lat : flat : geometry : planar", "lat : flat : lattice_type : simple_cubic",
        "lat : flat : bondlength : 3e-10",
        "lat : flat : lowerbound_x : surface", "lat : flat : upperbound_x : mirror",
        "lat : flat : lowerbound_y : periodic", "lat : flat : upperbound_y : periodic",
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : X : freedom : pinned", "mon : X : pinned_range : firstlayer",
        "mon : A : freedom : free", "mon : W : freedom : free",
        "mon : Na : freedom : free", "mon : Na : valence : 1", "mon : Cl : freedom : free", "mon : Cl : valence : -1",
        "mon : A : chi_S : -1", "mon : X : chi_W : 0.5",
        "state : AH : mon : A", "state : AH : valence : 0", "state : AM : mon : A", "state : AM : valence : -1",
        "state : H3O : mon : W", "state : H3O : valence : 1", "state : H2O : mon : W", "state : H2O : valence : 0",
        "state : OH : mon : W", "state : OH : valence : -1", f"state : H3O : alphabulk : {h3o}",
        "state : AH : chi_H2O : 0.8",
        "reaction : weak : equation : 1(AH) + 1(H2O) = 1(AM) + 1(H3O)", "reaction : weak : pK : 6",
        "reaction : auto : equation : 2(H2O) = 1(OH) + 1(H3O)", "reaction : auto : pK : 14",
        f"mol : pol : composition : (X)1(A){N - 1}", "mol : pol : freedom : restricted", f"mol : pol : n : {n!r}",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent",
        "mol : Na : composition : (Na)1", "mol : Na : freedom : neutralizer",
        "mol : Cl : composition : (Cl)1", "mol : Cl : freedom : free", "mol : Cl : phibulk : 0.01",
        "newton : isaac : method : DIIS", f"newton : isaac : tolerance : {tol}",
        f"newton : isaac : iterationlimit : {itlim}", "newton : isaac : deltamax : 0.1", "newton : isaac : m : 10",
    ]) + "\n"


def run_weak2d(args) -> dict:
    """On one GPU: the weak-polyacid brush with internal states (weak2d_text,
    100×100, A_200, sigma 0.05).  A step is `--iters` DIIS iterations from a
    seeded field x ~ U(-0.01, 0.01) (ψ and the state blocks included); its
    time is the context stream's CUDA-event interval; L2 is flushed between
    steps.  value = DIIS iterations per second, FP64 propagators; the FP32
    arm (one exponent per lattice row, FP64 composition, residual, Poisson
    update and DIIS) beside it.  Also the max |Δφ| of one residual at the
    seeded field against the CPU oracle, and the oracle's time for that
    residual on one core."""
    import torch
    from namics_gb300 import build as b
    b.build_product()
    from namics_gb300 import NM_FP32, NM_FP64, Context, Plan
    nx = ny = args.n2d
    N, sigma = 200, 0.05
    plan = Plan(weak2d_text(nx, ny, N, sigma * ny, itlim=args.iters))
    x0h = np.random.default_rng(SEED + 11).uniform(-0.01, 0.01, size=plan.iv)
    x0 = torch.from_numpy(x0h).cuda()
    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device="cuda")
    out = {}
    for prec, name in ((NM_FP64, "fp64"), (NM_FP32, "fp32")):
        st = torch.cuda.Stream()
        ctx = Context(plan, prec, stream=st.cuda_stream)
        xw = torch.empty_like(x0)
        times, its, res = [], [], None
        clocks = ClockSampler(0)
        with clocks:
            for k in range(args.warmup + args.steps):
                flush.zero_()
                xw.copy_(x0)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                res = ctx.solve_dev(xw.data_ptr())
                e1.record(st)
                e1.synchronize()
                if k >= args.warmup:
                    times.append(e0.elapsed_time(e1))
                    its.append(res.iterations + 1)
        ms = statistics.mean(times)
        n_its = statistics.mean(its)
        gd = torch.zeros_like(x0)
        ctx.residual_dev(x0.data_ptr(), gd.data_ptr())
        out[name] = {"ms_per_step": ms, "residuals_per_step": n_its, "iterations_per_s": 1000.0 * n_its / ms,
                     "residual_after_step": res.residual, "launches": ctx.launch_count(),
                     "clocks": clocks.summary(), "phi": ctx.field(0), "phi_states": ctx.field(9)}
        ctx.close()
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        b.build_oracle()
        from orc import Oracle
        orc = Oracle(plan)
        t0 = time.perf_counter()
        rc, _ = orc.residual(x0h)
        t_orc = time.perf_counter() - t0
        if rc == 0:
            mask = np.tile(plan.interior_mask(), plan.n_seg)
            po, ps = orc.field(0)[mask], orc.field(9)
            smask = np.tile(plan.interior_mask(), plan.c.n_state)
            for name in out:
                out[name]["max_abs_dphi_vs_oracle"] = float(np.max(np.abs(out[name]["phi"][mask] - po)))
                out[name]["max_abs_dphi_states_vs_oracle"] = float(
                    np.max(np.abs(out[name]["phi_states"][smask] - ps[smask])))
            out["cpu_residual_seconds"] = t_orc
    f32, f64 = out["fp32"], out["fp64"]
    updates = float(plan.segment_updates())
    strip = lambda d: {k: v for k, v in d.items() if k not in ("phi", "phi_states")}
    return {
        "metric": f"SCF DIIS iterations/s, {nx}x{ny} weak-polyacid brush with internal states and reactions "
                  "(FP64 GPU; FP32 propagators beside it)",
        "value": f64["iterations_per_s"], "unit": "iterations/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": f64["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded field)",
        "config": {"workload": f"{nx}x{ny} planar weak-polyacid brush, (X)1(A){N - 1} pinned, sigma {sigma}, "
                               "states AH/AM and H3O+/H2O/OH-, pK 6 and 14, H3O+ fraction 1e-7, Na neutraliser, "
                               "Cl phi_b 0.01",
                   "iteration_blocks": plan.c.n_it, "iterations_per_step": args.iters,
                   "l2": "flushed between steps (256 MB write)", "segment_site_updates_per_residual": updates},
        "updates_per_s": updates * f64["iterations_per_s"],
        "fp32": strip(f32), "fp64_gpu": dict(strip(f64), value=f64["iterations_per_s"], unit="iterations/s"),
        "cpu_residual_seconds": out.get("cpu_residual_seconds"),
    }


def run_served(args) -> dict:
    """A Poisson request stream served on one GPU by nm_server
    (continuous batching: 1-gradient requests go into the streaming work
    loop, admitted into resident CTAs as slots free up; the others get a
    device context each on W worker streams, admitted by device footprint).
    Mix: 70% 1-D brushes/stars drawn like the batched workload,
    25% 2-D 100×100 (A)200 adsorption, 5% 3-D 64³ (A)20(B)20 melts at
    chi 0.4, all from seeded fields.  Reported: converged solves/s over the
    span from the first submit to the last completion, p50/p99 of the
    submit-to-completion time, for FP32 propagators and for an FP64 server;
    and the plain FP64 GPU path: the same requests solved one at a time."""
    import torch  # noqa: F401  (device initialisation)
    from namics_gb300 import build as b
    b.build_product()
    from namics_gb300 import NM_FP32, NM_FP64, Plan, Server
    rng = np.random.default_rng(SEED + 7)
    n_req = args.requests
    brush_texts = workload(max(1, int(0.7 * n_req) + 8))
    kinds = rng.choice(3, size=n_req, p=[0.70, 0.25, 0.05])
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=n_req))
    ads, melt = Plan(ads2d_text()), Plan(melt3d_small_text())
    reqs, bi = [], 0
    for k in kinds:
        if k == 0:
            p = Plan(brush_texts[bi]); bi += 1
            x = rng.uniform(*FIELD, size=p.iv)
        elif k == 1:
            p = ads
            x = rng.uniform(-0.01, 0.01, size=p.iv)
        else:
            p = melt
            u = rng.uniform(-0.1, 0.1, size=p.M)
            x = np.concatenate([u, -u])
        reqs.append((int(k), p, x))
    out = {}
    sweeps = getattr(args, "context_sweeps", 0)
    arms = ((NM_FP32, "fp32"),) if args.no_fp64 else ((NM_FP32, "fp32"), (NM_FP64, "fp64"))
    for prec, name in arms:
        srv = Server(precision=prec, workers=args.workers, max_batch=64, memory_budget=64 << 30,
                     context_sweeps=sweeps)
        t0 = time.perf_counter()
        ids = []
        for (k, p, x), ta in zip(reqs, arrivals):
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            ids.append((k, srv.submit(p, x)))
        lat, ok, by_kind = [], 0, {0: [], 1: [], 2: []}
        for k, rid in ids:
            res, _, sec = srv.wait(rid)
            lat.append(sec)
            by_kind[k].append(sec)
            ok += res.status == 0
        span = time.perf_counter() - t0
        launches = srv.launch_count()
        srv.close()
        lat = np.array(lat) * 1e3
        out[name] = {"value": ok / span, "unit": "solves/s", "converged": int(ok), "requests": n_req,
                     "span_s": span, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "p50_ms_by_kind": {kn: (float(np.percentile(np.array(v) * 1e3, 50)) if v else None)
                                        for kn, v in zip(("brush1d", "ads2d", "melt3d"), by_kind.values())},
                     "p99_ms_by_kind": {kn: (float(np.percentile(np.array(v) * 1e3, 99)) if v else None)
                                        for kn, v in zip(("brush1d", "ads2d", "melt3d"), by_kind.values())},
                     "requests_by_kind": {kn: len(v) for kn, v in zip(("brush1d", "ads2d", "melt3d"),
                                                                     by_kind.values())},
                     "gpu_launches": launches}
    # the plain FP64 GPU path: the same requests one after another, each in a
    # device context with FP64 propagators and the host-driven DIIS loop
    from namics_gb300 import Context
    if not args.no_fp64:
        t0 = time.perf_counter()
        ok = 0
        for k, p, x in reqs:
            c = Context(p, NM_FP64)
            r, _ = c.solve_host(x.copy(), want_phi=False)
            ok += r.status == 0
            c.close()
        span = time.perf_counter() - t0
        out["fp64_plain"] = {"value": ok / span, "unit": "solves/s", "converged": int(ok), "requests": n_req,
                             "span_s": span, "what": "the same requests one at a time (no server), FP64 "
                                                     "propagators, DIIS with a host synchronisation per iteration"}
    f32 = out["fp32"]
    line = {
        "metric": METRIC, "value": f32["value"], "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": f32["span_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded request stream)",
        "config": {"workload": f"Poisson request stream, {args.rate:g} requests/s, {n_req} requests; 70% "
                               "1-D brushes/stars as in the batched workload, 25% 2-D 100x100 (A)200 adsorption, 5% 3-D 64^3 (A)20(B)20 melts",
                   "workers": args.workers, "max_batch": 64, "memory_budget_gb": 64,
                   "context_sweeps": sweeps},
        "latency": {"p50_ms": f32["p50_ms"], "p99_ms": f32["p99_ms"], "what": "submit to completion"},
        "fp32": f32, "fp64_gpu": out.get("fp64"), "fp64_plain": out.get("fp64_plain"),
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 GPU comparison")
    ap.add_argument("--workload", default="brush1d", choices=["brush1d", "melt3d", "cyl2d", "weak2d", "served"],
                    help="brush1d: 512 batched 1-D brushes/stars, the headline; melt3d: 128³ melt (DIIS iterations/s); "
                         "cyl2d: 200×200 charged cylindrical brushes at two chi values (DIIS iterations/s); "
                         "weak2d: 2-D weak-polyacid brush with internal states (DIIS iterations/s); "
                         "served: Poisson request stream of mixed solves")
    ap.add_argument("--n2d", type=int, default=200, help="cyl2d, weak2d: lattice edge")
    ap.add_argument("--no-solve", action="store_true", help="cyl2d: skip the timed full solves")
    ap.add_argument("--rate", type=float, default=20.0, help="served: arrivals per second")
    ap.add_argument("--requests", type=int, default=200, help="served: requests in the stream")
    ap.add_argument("--workers", type=int, default=8, help="served: concurrent solves")
    ap.add_argument("--context-sweeps", type=int, default=0,
                    help="served: options of the 2-D/3-D request contexts (bit mask: 1 persistent 2-D sweeps, "
                         "2 cluster sweeps of small FP32 3-D boxes, 4 device-resident solve loop)")
    ap.add_argument("--iters", type=int, default=20, help="melt3d: DIIS iterations per step")
    ap.add_argument("--n3d", type=int, default=128, help="melt3d: box edge")
    ap.add_argument("--ckpt", type=int, default=10, help="melt3d: checkpoint stride of the FP32 arm (0: store all)")
    ap.add_argument("--instances", type=int, default=N_INSTANCES)
    ap.add_argument("--no-others", action="store_true",
                    help="brush1d: skip the short runs of the melt, cylinder, weak-polyacid and served workloads")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "melt3d":
        print(json.dumps(run_melt3d(args)), flush=True)
        return
    if args.workload == "served":
        print(json.dumps(run_served(args)), flush=True)
        return
    if args.workload == "cyl2d":
        print(json.dumps(run_cyl2d(args)), flush=True)
        return
    if args.workload == "weak2d":
        print(json.dumps(run_weak2d(args)), flush=True)
        return
    run_brush1d(args)


def stream_fields(plans, steps: int, seed0: int):
    """Start fields of `steps` consecutive steps of the stream: every step
    solves the same instances from a fresh seeded field (step k: seed0 + k)."""
    return [x for k in range(steps) for x in fields(plans, seed=seed0 + k)]


def plain_fp64_sample(plans, xs, budget_s: float = 6.0, stream=None):
    """The plain FP64 GPU path: one solve at a time through a device context
    (nm_solve_dev: the reference's Solve loop, FP64 propagators, one problem
    on the whole GPU), over the first instances for about budget_s.  Returns
    converged solves/s and the sample."""
    import torch
    from namics_gb300 import NM_FP64, Context
    done, ok, t_gpu = 0, 0, 0.0
    t0 = time.perf_counter()
    for p, x in zip(plans, xs):
        if time.perf_counter() - t0 > budget_s:
            break
        ctx = Context(p, NM_FP64, stream=stream.cuda_stream if stream else None)
        xd = torch.from_numpy(x.copy()).cuda()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        st = stream or torch.cuda.current_stream()
        e0.record(st)
        r = ctx.solve_dev(xd.data_ptr())
        e1.record(st)
        e1.synchronize()
        t_gpu += e0.elapsed_time(e1) / 1000.0
        ctx.close()
        done += 1
        ok += r.status == 0
    return {"value": ok / t_gpu if t_gpu > 0 else None, "unit": UNIT, "converged": ok, "solves": done,
            "seconds": t_gpu, "what": "one solve at a time, device context, FP64 propagators, DIIS with a host "
                                      "sync per iteration (nm_solve_dev); first instances of the workload"}


def other_workloads(args) -> dict:
    """Short runs of the other workloads, measured in the same process: the
    128³ melt (DIIS iterations/s, FP32 propagators checkpointed every 10
    segments vs plain FP64), the 200×200 charged cylindrical brushes at both
    χ (iterations/s, FP32 vs FP64, |Δφ| of one residual against the oracle)
    and the served Poisson mix of 1-D, 2-D and 3-D requests (converged
    solves/s, p50/p99, FP32 server vs plain-FP64 server).  Each reports its
    own line's fields without the per-line contract keys."""
    import copy
    out = {}
    keep = ("metric", "value", "unit", "ms_per_step", "config", "roofline", "updates_per_s", "latency",
            "fp32", "fp32_full_storage", "fp32_autotuned", "fp64_gpu", "fp64_plain", "cpu_residual_seconds")
    runs = (("melt128", run_melt3d, dict(n3d=128, iters=5, steps=2, warmup=1, ckpt=10)),
            ("cylinder200", run_cyl2d, dict(n2d=200, iters=5, steps=2, warmup=1, no_solve=True)),
            ("weak_polyacid100", run_weak2d, dict(n2d=100, iters=5, steps=2, warmup=1)),
            ("served_mix", run_served, dict(rate=400.0, requests=200, workers=24)))
    for name, fn, over in runs:
        a = copy.copy(args)
        for k, v in over.items():
            setattr(a, k, v)
        try:
            d = fn(a)
            out[name] = {k: d[k] for k in keep if k in d}
        except Exception as e:  # a failure of one short run must not lose the headline line
            out[name] = {"error": f"{type(e).__name__}: {e}"[:300]}
    return out


# DRAM bytes (read + write) per problem of the work loop on this workload,
# from an ncu capture of a 1024-problem launch: 32.01 + 47.16 GB
TRAFFIC_PER_PROBLEM = (32.01e9 + 47.16e9) / 1024


def run_brush1d(args) -> None:
    """The headline: a sustained stream of batched 1-D brush/star solves.

    Every step brings the 512 instances of the workload with a fresh seeded
    start field (step k draws its fields from seed SEED + 1 + k).  The K timed
    steps (K × 512 solves) go through ONE device-resident work loop
    (nm_batch_solve_dev): resident CTAs, one per slot, take the next problem
    from the queue as soon as their last one converged, so a long or
    non-converging solve holds one slot, not the step.  value = converged
    solves / time of the K steps; ms_per_step = that time / K."""
    ws, rank, local = dist_env()
    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from namics_gb300 import build as b
    if rank == 0:
        b.build_product()
        b.build_oracle()
    if ws > 1:
        dist.barrier()
    from namics_gb300 import NM_FP32, NM_FP64, Batch, Plan

    texts = workload(args.instances)
    plans = [Plan(t) for t in texts]
    K, W = args.steps, args.warmup
    prec = NM_FP32 if args.precision == "fp32" else NM_FP64
    stream = torch.cuda.Stream()
    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    xs = stream_fields(plans, K, SEED + 1)
    x0 = torch.from_numpy(np.concatenate(xs)).cuda()
    xw = torch.empty_like(x0)
    job = Batch(plans * K, prec, device=local, stream=stream.cuda_stream)
    # untimed warm-up: W steps of the same stream (their own seeds); the
    # autotuner picks the work loop's resident CTAs per SM on them
    tuning = None
    if W > 0:
        xwu = np.concatenate(stream_fields(plans, W, SEED + 1001))
        warm = Batch(plans * W, prec, device=local, stream=stream.cuda_stream)
        xwd = torch.from_numpy(xwu).cuda()
        tuning = warm.autotune(xwd.data_ptr())
        warm.solve_host(xwu)
        warm.close()
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        job.slots = tuning["ctas_per_sm"] * sms  # the tuned CTAs per SM (K×512 problems: every slot fits)
    # timed: the K steps in one work loop, inputs resident in HBM, L2 flushed
    xw.copy_(x0)
    flush.zero_()
    launches0 = job.launch_count()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        its_all, res, st = job.solve_dev(xw.data_ptr())
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    total_ms = e0.elapsed_time(e1)
    launches = job.launch_count() - launches0
    queued, solving = job.timings()
    fp32_its = job.fp32_iterations() if prec == NM_FP32 else None
    ok = st == 0
    n_ok = int(ok.sum())
    latency = {"p50_ms": float(np.percentile(solving[ok] * 1e3, 50)) if ok.any() else None,
               "p99_ms": float(np.percentile(solving[ok] * 1e3, 99)) if ok.any() else None,
               "queue_wait_p50_ms": float(np.percentile(queued * 1e3, 50)),
               "queue_wait_p99_ms": float(np.percentile(queued * 1e3, 99)),
               "unit": "ms", "what": "per converged problem: time to convergence in its slot (device timer); "
                                     "queue wait from the work loop's start to the problem's start"}
    # roofline: algorithmic bytes of the propagator work of the launch
    updates = 0.0
    per_it = [p.segment_updates() for p in plans]
    for i in range(len(its_all)):
        updates += per_it[i % len(plans)] * (int(its_all[i]) + 1)
    # the same stream with FP64 propagators throughout (same work loop)
    fp64 = None
    if prec == NM_FP32 and not args.no_fp64:
        K64 = max(1, min(K, 4))
        j64 = Batch(plans * K64, NM_FP64, device=local, stream=stream.cuda_stream)
        x64 = torch.from_numpy(np.concatenate(xs[:K64 * len(plans)])).cuda()
        flush.zero_()
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        _, _, st64 = j64.solve_dev(x64.data_ptr())
        a1.record(stream)
        a1.synchronize()
        ms64 = a0.elapsed_time(a1)
        n64 = int((st64 == 0).sum())
        fp64 = {"value": n64 / (ms64 / 1000.0), "unit": UNIT, "ms_per_step": ms64 / K64, "converged": n64,
                "steps": K64, "what": "the same stream and work loop, FP64 propagators throughout"}
        j64.close()
    plain64 = None
    if rank == 0 and not args.no_fp64:
        plain64 = plain_fp64_sample(plans, xs[:len(plans)], budget_s=6.0, stream=stream)
    # end to end through the C ABI with host buffers: the K steps' fields in,
    # solved fields out, copies inside the timed region
    xh = np.concatenate(xs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    job.solve_host(xh)
    e2e_s = time.perf_counter() - t0
    nbytes = xh.nbytes
    ms, e2e_s, n_all = reduce_over_ranks(total_ms, e2e_s, n_ok)
    value = n_all / (ms / 1000.0)
    bpu = B_PER_UPDATE_FP32 if prec == NM_FP32 else B_PER_UPDATE_FP64
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = updates * bpu / (total_ms / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if prec == NM_FP32 else "f64",
        "data": "synthetic (seeded brush/star instances, a fresh seeded start field every step)",
        "config": {"workload": "stream of batched 1-gradient brushes/stars: 512 seeded instances per step "
                               "(n_layers U{50..400}, N U{20..500}, sigma U[0.01,0.1], chi U[0,1], 10% 3-arm "
                               "stars), each step from fresh seeded fields; the K steps in one device-resident "
                               "work loop",
                   "instances_per_step": args.instances, "solves": len(its_all) * ws, "converged": n_all,
                   "precision": args.precision, "slots": job.slots,
                   "autotuned": tuning,
                   "iterations_mean": float(np.mean(its_all)), "iterations_max": int(np.max(its_all)),
                   "fp32_residuals_mean": float(np.mean(fp32_its)) if fp32_its is not None else None,
                   "segment_site_updates": updates,
                   "l2": "flushed once before the timed region (256 MB write); the K steps' inputs "
                         f"({nbytes / 1e6:.0f} MB of fields) are written to HBM before it",
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": TRAFFIC_PER_PROBLEM * len(its_all),
                     "note": f"{bpu:.0f} B per segment-site update x updates / work-loop time; peak of measured "
                             "(MEASURED_PEAKS.json hbm_gbs, burst copy); traffic: a constant from one ncu capture "
                             f"of this work loop ({TRAFFIC_PER_PROBLEM / 1e6:.1f} MB of DRAM reads + writes per "
                             "problem, the same at 512 and 1024 problems a launch) times the launch's problems, "
                             "not measured in this run"},
        "e2e": {"value": n_all / e2e_s, "unit": UNIT, "h2d_bytes_per_step": nbytes * ws // K,
                "d2h_bytes_per_step": nbytes * ws // K},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "latency": latency,
        "fp64_gpu": fp64,
        "fp64_gpu_unbatched": plain64,
    }
    if rank == 0 and not args.no_cpu and ws == 1:
        line["cpu_baseline"] = cpu_baseline(texts, xs[:len(plans)], budget_s=15.0)
    if rank == 0 and ws == 1 and not args.no_others:
        line["other_workloads"] = other_workloads(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
