#!/usr/bin/env python
"""Benchmark: particle-steps/s of the 320k-fluid-particle 2D dam break on GB300.

Workload (one "step" = one ``ForwardTime(dt)`` of the whole scene): a 0.2 m x
0.4 m water column at l0 = 5e-4 m (320,000 fluid particles) in a 0.8 m x 0.6 m
tank with 3 wall + 2 dummy layers (340,050 particles in all), the reference's
stock scheme (higher-order source and Laplacian, error-compensating source,
dynamic stabilisation, space potential particles) with one radius r_e = 4.0 l0
(PPE with ~45 nonzeros per row),
dt = 2.5e-5 s, PPE solved to |b - A x| <= 1e-8 |b|.  The data
are synthetic (seeded lattice scene); the state and the CSR/ELL matrix exceed L2,
and L2 is also flushed (512 MiB written, then read back) between timed steps.

Output: one JSON line.  ``value`` is whole-job particle-steps/s with the state
resident in HBM (CUDA events on the library's stream around each step); ``e2e``
is the same metric through the public C ABI with host buffers (host-to-device
copy of the full particle state, the step, device-to-host copy of the result),
over the same simulation steps (it restarts from the state the timed steps started
from, since later steps of the dam break need more PPE iterations);
``roofline`` reports the PPE solver's SpMV kernel (the dominant kernel) against
the measured HBM bandwidth; ``cpu_baseline`` times the CPU restatement of the
reference step (OpenMP, all host cores) on a bounded sample of the same scene.
Further blocks: ``ppe_solvers_same_state`` (every PPE solver from one snapshot),
``method_variants`` (GC, explicit pressure, and a 104k-particle 3D dam break),
``configs`` (the other configurations: throughput and SpMV GB/s, cache-resident
matrices tagged) and ``batched`` (256 independent scenes in one handle).

``--impl reference`` times that CPU path alone (rank 0 only) on the same
workload and metric, over the same simulation steps (``--warmup`` untimed steps
from the initial state, then ``--steps`` timed ones).  The headline solver is the
multigrid-preconditioned mixed-precision CG (``--solver mg``); the learned solver's
result stands beside it in ``ppe_solvers_same_state``.  With ``--gpus N`` (one process per GPU under torchrun)
every rank advances its own independent replica of the scene (replicas only: the
step has no data-parallel exchange), and ``value`` sums all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s, 320k dam break"
METRIC_FULL = METRIC + "; PPE ms to 1e-8 rel: learned vs plain CG"
UNIT = "particle-steps/s"
WORKLOAD = ("2D dam break, 320,000 fluid + 20,050 wall/dummy particles, l0=5e-4 m, reference MPS scheme "
            "(HS, HL, ECS, DS, SPP), re=4.0 l0, dt=2.5e-5 s")


def workload_config(particles: int, world: int) -> dict:
    """The `config` block, identical in both arms."""
    return {"workload": WORKLOAD, "particles": particles, "ppe_tolerance": "|b-Ax| <= 1e-8 |b|",
            "l2": "GPU arm: L2 flushed between timed steps (512 MiB written, then read back); working set > L2 in both arms",
            "parallelism": "replicas" if world > 1 else "single GPU"}
FALLBACK_HBM_GBS = 6800.0
FLUSH_BYTES = 512 << 20
SOLVERS = {"cg64": 0, "mixed": 1, "mg": 3, "learned": 2}
SOLVER_DESC = {0: "FP64 CG (reference algorithm)", 1: "FP32 CG + FP64 reliable updates",
               3: "FP32 CG preconditioned by the cell multigrid + FP64 reliable updates",
               2: "multigrid FP32 CG + FP64 reliable updates, learned initial guess and Jacobi scale"}


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--solver", choices=("cg64", "mixed", "mg", "learned"), default="mg")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the same-state comparison of the PPE solvers")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched 256-scene workload")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched workload and print its JSON (for profilers)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0,
                    help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cg-launch", choices=("graph", "host", "persistent"), default="graph",
                    help="host: CG kernels launched one by one (profilers cannot see kernels "
                         "inside conditional CUDA graphs)")
    ap.add_argument("--profile-scene", choices=("c2", "c1"), default="c2",
                    help="with --profile-steps: the 320k dam break (c2) or the 80k hydrostatic tank (c1)")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only run --warmup + this many steps and exit (for ncu)")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


# --------------------------------------------------------------- clock sampler
class ClockSampler:
    """Samples SM clock and throttle reasons with nvidia-smi during a timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power = [], [], []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU baseline
def cpu_model() -> str:
    """The host CPU's model name (lscpu on Arm hosts, whose /proc/cpuinfo names none)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        fields = dict(line.split(":", 1) for line in out.splitlines() if ":" in line)
        name = fields.get("Model name", "").strip()
        vendor = fields.get("Vendor ID", "").strip()
        if name:
            return (vendor + " " + name).strip()
    except (OSError, subprocess.SubprocessError, ValueError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


def cpu_baseline(scene, params, dt, budget_s: float, warmup: int = 0, max_steps: int | None = None) -> dict:
    """The CPU restatement of the reference step (OpenMP, all host threads): `warmup`
    untimed steps from the scene's initial state, then timed steps until `max_steps` or
    the time budget."""
    from oracle import build_oracle
    from oracle import oracle as orc

    build_oracle.build()
    o = orc.Oracle(params, openmp=True)
    o.add_scene(scene)
    threads = orc.num_threads(True)
    for _ in range(warmup):
        o.forward_time(dt)
    times, its = [], []
    t_all = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        o.forward_time(dt)
        times.append(time.perf_counter() - t0)
        its.append(o.stats()["cg_iterations"])
        if max_steps is not None and len(times) >= max_steps:
            break
        if max_steps is None and (time.perf_counter() - t_all + times[-1] > budget_s or len(times) >= 50):
            break
    n_active = int((o.particles()["type"] != 3).sum())
    sec = sum(times)
    return {"value": n_active * len(times) / sec, "unit": UNIT, "cores": threads, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": "steps %d-%d of the same scene (%d untimed before them), %.1f s of CPU time; "
                      "FP64 CG, %.0f iterations per step" % (warmup + 1, warmup + len(times), warmup, sec,
                                                             statistics.mean(its)),
            "seconds_per_step": sec / len(times), "cg_iterations_per_step": statistics.mean(its)}


def reduce_max(values, dist):
    """Max over ranks of per-rank timings: the slowest replica sets the job's time."""
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    buf = torch.tensor(list(values), dtype=torch.float64, device=dev)
    dist.all_reduce(buf, op=dist.ReduceOp.MAX)
    return buf.tolist()


def job_value(particles_per_replica: int, steps: int, world: int, total_ms: float) -> float:
    """Whole-job particle-steps/s: every rank advances its own replica of the scene."""
    return particles_per_replica * steps * world / (total_ms * 1e-3)


def load_peak() -> tuple[float, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def load_traffic(key: str, alg_bytes: float):
    """DRAM bytes per launch of the SpMV kernel from the committed ncu capture, scaled from
    the captured launch to this launch by algorithmic bytes (the matrix grows a little as
    the dam breaks); None without a capture for this solver."""
    path = os.path.join(ROOT, "profiles", "spmv_traffic.json")
    try:
        with open(path) as f:
            rec = json.load(f).get(key)
    except (OSError, ValueError):
        return None
    if not rec:
        return None
    return rec["dram_bytes"] * alg_bytes / rec["algorithmic_bytes"]


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world, local_rank):
    from openmps_gb300 import _abi as abi
    from openmps_gb300 import build as gpu_build
    from openmps_gb300 import scenes
    from openmps_gb300.computer import Computer

    gpu_build.build()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist  # noqa: F811

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    solver = SOLVERS[args.solver]
    scene = scenes.config_c1() if (args.profile_steps > 0 and args.profile_scene == "c1") else scenes.config_c2()
    dt = scene.meta["dt"]
    launch = {"graph": abi.CG_LAUNCH_GRAPH, "host": abi.CG_LAUNCH_HOST,
              "persistent": abi.CG_LAUNCH_PERSISTENT}[args.cg_launch]
    params = scene.params(solver=solver, criterion=abi.CRIT_RHS, eps=1e-8, cg_launch=launch)
    comp = Computer(params, device=local_rank)
    if solver == abi.SOLVER_LEARNED:
        from openmps_gb300 import learned

        comp.learned_set_weights(learned.load())
    comp.add_scene(scene)

    for _ in range(max(args.warmup, 0)):
        comp.forward_time(dt)
    if args.profile_steps > 0:
        for _ in range(args.profile_steps):
            comp.forward_time(dt)
        st = comp.stats()
        print(json.dumps({"profile_steps": args.profile_steps, "cg_iterations": st["cg_iterations"],
                          "ppe_nnz": st["ppe_nnz"], "kernel_launches": st["kernel_launches"]}))
        return
    n_active = comp.count - comp.stats()["disabled"]

    def barrier():
        if dist is not None:
            dist.barrier()

    # the state the timed steps start from: the end-to-end steps start from it too, so
    # both time the same steps of the simulation (the dam break gets harder as it runs)
    start_state = comp.particles()

    # ---- device-resident timed region
    sampler = ClockSampler(local_rank)
    launches0 = comp.stats()["kernel_launches"]
    iters = []
    barrier()
    comp.synchronize()
    sampler.start()
    total_ms = 0.0
    for _ in range(args.steps):
        comp.flush_l2(FLUSH_BYTES)
        comp.event_record(0)
        comp.forward_time(dt)
        comp.event_record(1)
        total_ms += comp.event_elapsed(0, 1)
        iters.append(comp.stats()["cg_iterations"])
    comp.synchronize()
    barrier()
    clocks = sampler.stop()
    launches = comp.stats()["kernel_launches"] - launches0
    n_active = comp.count - comp.stats()["disabled"]
    relres = comp.stats()["cg_true_relres"]

    # ---- end to end through the C ABI with pinned host buffers
    try:
        import torch

        pin = lambda n, dt_: torch.empty(n, dtype=dt_, pin_memory=True).numpy()
        import numpy as np

        host = {"type": pin(comp.count, torch.int32)}
        for k in ("x", "z", "u", "w", "p", "n"):
            host[k] = pin(comp.count, torch.float64)
        pinned = True
    except Exception:  # torch missing or no pinned memory: pageable host arrays
        import numpy as np

        host = {"type": np.empty(comp.count, dtype=np.int32)}
        for k in ("x", "z", "u", "w", "p", "n"):
            host[k] = np.empty(comp.count)
        pinned = False
    order = ("type", "x", "z", "u", "w", "p", "n")
    for k in order:
        host[k][:] = start_state[k]
    h2d = d2h = sum(host[k].nbytes for k in order)
    barrier()
    e2e_ms = 0.0
    for _ in range(args.steps):
        comp.flush_l2(FLUSH_BYTES)
        comp.event_record(2)
        comp.set_particles(*[host[k] for k in order])
        comp.forward_time(dt)
        comp.get_particles_into(*[host[k] for k in order])
        comp.event_record(3)
        e2e_ms += comp.event_elapsed(2, 3)
    barrier()

    # ---- stage breakdown (one extra step with per-stage events)
    comp.set_stage_timing(True)
    comp.forward_time(dt)
    stage_ms = {k: round(v, 3) for k, v in comp.stats()["stage_ms"].items()}
    comp.set_stage_timing(False)

    # ---- the PPE solvers on the same state (a few steps each from a snapshot)
    compare = variants = sweep = None
    if not args.no_compare and rank == 0:
        compare = compare_solvers(comp, scene, dt, local_rank)
        variants = method_variants(comp, scene, dt, local_rank)
        sweep = config_sweep(local_rank, load_peak()[0])

    # ---- the batched workload: 256 uneven dam breaks in one handle
    batched = None
    if not args.no_batch and rank == 0:
        batched = batched_workload(local_rank, args.batch_scenes, steps=max(2, min(args.steps, 10)))

    # ---- roofline of the dominant kernel (the solver's SpMV), timed alone
    st = comp.stats()
    nnz = st["ppe_nnz"]
    n = comp.count
    spmv_solver = abi.SOLVER_MIXED_MG if solver == abi.SOLVER_LEARNED else solver
    spmv_ms = comp.bench_spmv(spmv_solver, reps=20, flush_bytes=FLUSH_BYTES)
    # algorithmic bytes of one launch, from the library (it knows the FP32 layout)
    alg_bytes = comp.spmv_bytes(spmv_solver)
    if solver == abi.SOLVER_CG64:
        key, kernel = "cg64", "k_cg_spmv_dot"
    elif solver == abi.SOLVER_MIXED:
        key, kernel = "mixed", "k_mx_spmv"
    else:  # preconditioned: also reads u (own row) next to r
        key, kernel = "mg", "k_pmx_spmv"
    spmv64_ms = comp.bench_spmv(abi.SOLVER_CG64, reps=20, flush_bytes=FLUSH_BYTES)
    peak, peak_kind = load_peak()
    achieved = alg_bytes / (spmv_ms * 1e-3) / 1e9
    traffic = load_traffic(key, alg_bytes)
    alg64 = comp.spmv_bytes(abi.SOLVER_CG64)
    achieved64 = alg64 / (spmv64_ms * 1e-3) / 1e9

    # ---- reduce over ranks (max time)
    t_steps, t_e2e = total_ms, e2e_ms
    if dist is not None:
        t_steps, t_e2e = reduce_max([t_steps, t_e2e], dist)
    value = job_value(n_active, args.steps, world, t_steps)
    e2e_value = job_value(n_active, args.steps, world, t_e2e)

    if rank != 0:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return

    line = {
        "metric": METRIC_FULL,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_steps / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if solver == abi.SOLVER_CG64 else "f64 (PPE iterations f32, f64 residual/refinement)",
        "ppe_solver": SOLVER_DESC[solver],
        "data": "synthetic (seeded lattice dam break)",
        "config": workload_config(n, world),
        "impl": "ours",
        "solver": args.solver,
        "active_particles": n_active,
        "ppe_nnz": nnz,
        "cg_iterations_per_step": statistics.mean(iters) if iters else None,
        "ppe_true_relres": relres,
        "stage_ms": stage_ms,
        "gpu_launches": launches,
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "pinned_host_buffers": pinned},
        "roofline": {"bound": "hbm", "kernel": kernel,
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": alg_bytes, "ms_per_launch": spmv_ms,
                     "spmv64": {"kernel": "k_cg_spmv_dot_staged", "ms_per_launch": spmv64_ms,
                                "algorithmic_bytes_per_launch": alg64, "achieved": achieved64,
                                "frac": achieved64 / peak, "traffic": load_traffic("cg64", alg64)}},
    }
    # the long blocks first; the compact solver comparison closes the line
    if sweep is not None:
        line["configs"] = sweep
    if variants is not None:
        line["method_variants"] = variants
    if batched is not None:
        line["batched"] = batched
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(scene, scene.params(criterion=abi.CRIT_RHS, eps=1e-8), dt,
                                            args.cpu_seconds, warmup=max(args.warmup, 0))
    if compare is not None:
        line["ppe_solvers_same_state"] = compare
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def compare_solvers(comp, scene, dt, device, steps=3):
    """Step and PPE-solve time of every solver from the same particle state (a snapshot
    of the timed run), `steps` steps each, with per-stage CUDA events."""
    from openmps_gb300 import _abi as abi
    from openmps_gb300 import learned
    from openmps_gb300.computer import Computer

    P = comp.particles()
    A = comp.aux()
    out = {}
    for name in ("cg64", "mixed", "mg", "learned"):
        sv = SOLVERS[name]
        c = Computer(scene.params(solver=sv, criterion=abi.CRIT_RHS, eps=1e-8), device=device)
        if sv == abi.SOLVER_LEARNED:
            c.learned_set_weights(learned.load())
        c.add_particles(P["type"], P["x"], P["z"], P["u"], P["w"], P["p"], P["n"])
        c.set_aux(A["n_without_spp"], A["ecs"], A["ox"], A["oz"])
        c.set_stage_timing(True)
        step_ms, solve_ms, its, fbs = [], [], [], 0
        for _ in range(steps):
            c.flush_l2(FLUSH_BYTES)
            c.event_record(0)
            c.forward_time(dt)
            c.event_record(1)
            step_ms.append(c.event_elapsed(0, 1))
            st = c.stats()
            solve_ms.append(st["stage_ms"]["solve"])
            its.append(st["cg_iterations"])
            fbs += st["fallback"]
            assert st["cg_true_relres"] <= 1e-8
        c.close()
        out[name] = {"step_ms": round(statistics.mean(step_ms), 3), "ppe_ms": round(statistics.mean(solve_ms), 3),
                     "iterations": round(statistics.mean(its), 1), "fp64_fallbacks": fbs}
    base = out["cg64"]
    for name, v in list(out.items()):
        v["step_x_vs_cg64"] = round(base["step_ms"] / v["step_ms"], 2)
        v["ppe_x_vs_cg64"] = round(base["ppe_ms"] / v["ppe_ms"], 2)
    out["note"] = ("one snapshot, %d steps per solver, L2 flushed before each step, PPE to 1e-8 |b|: cg64 = FP64 CG "
                   "(reference algorithm), mixed = FP32 CG + FP64 reliable updates (the FP64 CG finishes it when it "
                   "stalls), mg = mixed preconditioned by the cell multigrid, learned = mg started from the network's guess and Jacobi scale" % steps)
    return out


VARIANT_SOUND_SPEED = 28.0  # about ten times sqrt(2 g h) of the 0.4 m water column


def method_variants(comp, scene, dt, device, steps=3):
    """The workload's step with the other method flags, from the same snapshot: the GC
    corrective-matrix gradient (multigrid solver), and the explicit pressure (no PPE; its
    own CFL time step courant l0 / c) with and without GC.  Per-stage CUDA events."""
    from openmps_gb300 import _abi as abi
    from openmps_gb300.computer import Computer

    P = comp.particles()
    A = comp.aux()
    stock = abi.PRESET_REFERENCE
    l0 = scene.l0
    dt_explicit = 0.1 * l0 / VARIANT_SOUND_SPEED
    cases = {
        "stock_mg": (stock, dt),
        "gc_mg": (stock | abi.FLAG_GC, dt),
        "explicit": (stock | abi.FLAG_PRESSURE_EXPLICIT, dt_explicit),
        "explicit_gc": (stock | abi.FLAG_PRESSURE_EXPLICIT | abi.FLAG_GC, dt_explicit),
    }
    out = {}
    for name, (flags, step_dt) in cases.items():
        c = Computer(scene.params(solver=abi.SOLVER_MIXED_MG, criterion=abi.CRIT_RHS, eps=1e-8,
                                  flags=flags, sound_speed=VARIANT_SOUND_SPEED), device=device)
        c.add_particles(P["type"], P["x"], P["z"], P["u"], P["w"], P["p"], P["n"])
        c.set_aux(A["n_without_spp"], A["ecs"], A["ox"], A["oz"])
        c.set_stage_timing(True)
        step_ms, grad_ms, pres_ms = [], [], []
        for _ in range(steps):
            c.flush_l2(FLUSH_BYTES)
            c.event_record(0)
            c.forward_time(step_dt)
            c.event_record(1)
            step_ms.append(c.event_elapsed(0, 1))
            st = c.stats()["stage_ms"]
            grad_ms.append(st["gradient"])
            pres_ms.append(st["pressure"])
        c.close()
        ms = statistics.mean(step_ms)
        out[name] = {"flags": flags, "dt": step_dt, "step_ms": ms, "gradient_ms": statistics.mean(grad_ms),
                     "pressure_ms": statistics.mean(pres_ms), "particle_steps_per_s": scene.count / (ms * 1e-3)}
    out["note"] = ("same snapshot, %d steps each, L2 flushed before each step; explicit: c = %g m/s, "
                   "dt = courant l0 / c" % (steps, VARIANT_SOUND_SPEED))
    out["dim3"] = dim3_workload(device)
    return out


def config_sweep(device, peak, warmup=3, steps=5):
    """Throughput and SpMV bandwidth of the other configurations: C0 (the l0 = 0.01 dam
    break, 800 fluid), C1 (the 80,000-fluid hydrostatic tank) and the 320k dam break at
    the smaller radius r_e = 2.1 l0 (13 nonzeros per PPE row), each with the multigrid
    mixed-precision solver to
    |b - Ax| <= 1e-8 |b|, L2 flushed before every timed step.  The SpMVs are timed alone,
    L2 flushed before each launch; a matrix that fits in L2 is tagged, because there the
    GB/s exceed what HBM alone delivers when L2 is warm."""
    from openmps_gb300 import _abi as abi
    from openmps_gb300 import scenes
    from openmps_gb300.computer import Computer

    c2_one = scenes.config_c2()
    c2_one.meta["params"] = dict(c2_one.meta["params"], re_by_l0=2.1, re_lap_by_l0=0.0)
    cases = (("C0 dam break, 800 fluid, l0=1e-2 m, dt=5e-4 s", scenes.config_c0()),
             ("C1 hydrostatic tank, 80,000 fluid, l0=2.5e-3 m, dt=1e-4 s", scenes.config_c1()),
             ("C2 320k dam break at r_e = 2.1 l0, dt=2.5e-5 s", c2_one))
    out = []
    for name, sc in cases:
        dt = sc.meta["dt"]
        c = Computer(sc.params(solver=abi.SOLVER_MIXED_MG, criterion=abi.CRIT_RHS, eps=1e-8), device=device)
        c.add_scene(sc)
        for _ in range(warmup):
            c.forward_time(dt)
        ms, its = [], []
        for _ in range(steps):
            c.flush_l2(FLUSH_BYTES)
            c.event_record(0)
            c.forward_time(dt)
            c.event_record(1)
            ms.append(c.event_elapsed(0, 1))
            its.append(c.stats()["cg_iterations"])
        st = c.stats()
        n, nnz = sc.count, st["ppe_nnz"]
        b32 = c.spmv_bytes(abi.SOLVER_MIXED)
        b64 = c.spmv_bytes(abi.SOLVER_CG64)
        t32 = c.bench_spmv(abi.SOLVER_MIXED, reps=20, flush_bytes=FLUSH_BYTES)
        t64 = c.bench_spmv(abi.SOLVER_CG64, reps=20, flush_bytes=FLUSH_BYTES)
        c.close()
        out.append({"workload": name, "particles": n, "ppe_nnz": nnz, "ms_per_step": statistics.mean(ms),
                    "particle_steps_per_s": n / (statistics.mean(ms) * 1e-3),
                    "ppe_iterations": statistics.mean(its),
                    "spmv32": {"ms": t32, "gbs": b32 / (t32 * 1e-3) / 1e9, "frac": b32 / (t32 * 1e-3) / 1e9 / peak,
                               "bytes": b32, "l2_resident": b32 < 100e6},
                    "spmv64": {"ms": t64, "gbs": b64 / (t64 * 1e-3) / 1e9, "frac": b64 / (t64 * 1e-3) / 1e9 / peak,
                               "bytes": b64, "l2_resident": b64 < 100e6}})
    return out


def dim3_workload(device, warmup=2, steps=3):
    """A three-dimensional dam break (DIM3): a 0.1 x 0.2 x 0.2 m column in a 0.4 x 0.2 x 0.4 m
    box at l0 = 5 mm, the reference's stock method set at r_e = 2.4 l0 (Sample.xml), dt =
    2.5e-4 s, PPE to |b - Ax| <= 1e-8 |b| with the FP64 CG and the mixed-precision CG."""
    from openmps_gb300 import _abi as abi
    from openmps_gb300 import scenes
    from openmps_gb300.computer import Computer

    scene = scenes.dam_break3d(5e-3, water=(0.1, 0.2, 0.2), tank=(0.4, 0.2, 0.4))
    scene.meta["params"] = dict(scenes.STOCK_PHYSICS, re_by_l0=2.4, re_lap_by_l0=0.0, max_dt=1.0)
    dt = 2.5e-4
    out = {"workload": "3D dam break, %d fluid + %d wall/dummy particles, l0=5e-3 m, HS HL ECS DS SPP, "
                       "re=2.4 l0, dt=%g s" % (int((scene.type == 0).sum()), int((scene.type != 0).sum()), dt),
           "particles": scene.count}
    for name, solver in (("cg64", abi.SOLVER_CG64), ("mixed", abi.SOLVER_MIXED)):
        c = Computer(scene.params(solver=solver, criterion=abi.CRIT_RHS, eps=1e-8), device=device)
        c.add_particles3(*scene.arrays3())
        for _ in range(warmup):
            c.forward_time(dt)
        c.set_stage_timing(True)
        step_ms, ppe_ms, its = [], [], []
        for _ in range(steps):
            c.flush_l2(FLUSH_BYTES)
            c.event_record(0)
            c.forward_time(dt)
            c.event_record(1)
            step_ms.append(c.event_elapsed(0, 1))
            st = c.stats()
            ppe_ms.append(st["stage_ms"]["solve"])
            its.append(st["cg_iterations"])
        out[name] = {"step_ms": statistics.mean(step_ms), "ppe_ms": statistics.mean(ppe_ms),
                     "iterations": statistics.mean(its), "ppe_nnz": c.stats()["ppe_nnz"],
                     "particle_steps_per_s": scene.count / (statistics.mean(step_ms) * 1e-3)}
        c.close()
    return out


def batched_workload(device, nscenes, steps):
    """Particle-steps/s of `nscenes` independent dam breaks (width U[0.1, 0.3] m, height
    U[0.2, 0.5] m, l0 = 5 mm, seeded) advanced together: the first step autotunes the
    batched solve, the timed steps replay the captured per-step graph."""
    from openmps_gb300 import _abi as abi
    from openmps_gb300 import scenes as sc_mod
    from openmps_gb300.computer import Batch

    l0 = 5e-3
    dt = l0 / 20.0
    scs = []
    for k in range(nscenes):
        s = sc_mod.batch_scene(k, seed=20261203, l0=l0)
        s.meta["params"] = dict(sc_mod.STOCK_PHYSICS, eps=1e-8, max_dt=dt)
        scs.append(s)
    prm = scs[0].params(solver=abi.SOLVER_MIXED_MG, criterion=abi.CRIT_RHS, eps=1e-8)
    b = Batch(prm, scs, device=device)
    b.forward(dt, 1)  # autotune + first step
    b.forward(dt, 2)  # capture + warm-up
    b.synchronize()
    b.flush_l2(FLUSH_BYTES)
    b.event_record(0)
    b.forward(dt, steps)
    b.event_record(1)
    ms = b.event_elapsed(0, 1)
    particles = int(sum(s.count for s in scs))
    fluid = int(sum(int((s.type == abi.TYPE_FLUID).sum()) for s in scs))
    its = [b.scene_stats(k) for k in range(nscenes)]
    out = {
        "workload": "%d independent 2D dam breaks, l0=5e-3 m, columns U[0.1,0.3] x U[0.2,0.5] m in "
                    "0.8 x 0.6 m tanks, reference MPS scheme, dt=%.2e s" % (nscenes, dt),
        "scenes": nscenes, "particles": particles, "fluid_particles": fluid,
        "fluid_per_scene_min": int(min((s.type == abi.TYPE_FLUID).sum() for s in scs)),
        "fluid_per_scene_max": int(max((s.type == abi.TYPE_FLUID).sum() for s in scs)),
        "steps": steps, "ms_per_step": ms / steps,
        "value": particles * steps / (ms * 1e-3), "unit": UNIT,
        "ppe_iterations_mean": statistics.mean(t["iterations"] for t in its),
        "ppe_iterations_max": max(t["iterations"] for t in its),
        "fallbacks": int(sum(t["fallback"] for t in its)),
        "max_true_relres": max(t["true_relres"] for t in its),
        "tuning": b.tuning(),
        "launch": "per step one replay of a captured CUDA graph: stage kernels over all scenes + "
                  "one persistent block-per-scene PPE solve",
    }
    b.close()
    return out


# ------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    """The CPU restatement of the reference step (OpenMP, all host threads), over the same
    simulation steps as the GPU arm: `--warmup` untimed steps from the initial state, then
    `--steps` timed ones."""
    if rank != 0:
        return
    from openmps_gb300 import _abi as abi
    from openmps_gb300 import scenes

    scene = scenes.config_c2()
    dt = scene.meta["dt"]
    params = scene.params(criterion=abi.CRIT_RHS, eps=1e-8)
    warmup = max(args.warmup, 0)
    cb = cpu_baseline(scene, params, dt, budget_s=1e9, warmup=warmup, max_steps=max(1, args.steps))
    line = {
        "metric": METRIC_FULL, "value": cb["value"], "unit": UNIT, "n_gpus": world, "steps": max(1, args.steps),
        "warmup": warmup, "ms_per_step": cb["seconds_per_step"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lattice dam break)",
        "config": workload_config(scene.count, world),
        "impl": "reference",
        "solver": "cg64",
        "note": "the reference (header-only C++ with Boost/ViennaCL) cannot be built here; this arm runs its "
                "C++ restatement (the oracle) with OpenMP on all host cores",
        "cpu_baseline": {"value": cb["value"], "unit": UNIT, "cores": cb["cores"], "kind": cb["kind"],
                         "cpu_model": cb["cpu_model"], "sample": cb["sample"]},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    rank, world, local_rank = dist_env()
    if args.batch_only:
        from openmps_gb300 import build as gpu_build

        gpu_build.build()
        print(json.dumps(batched_workload(local_rank, args.batch_scenes, steps=max(2, args.steps))), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
