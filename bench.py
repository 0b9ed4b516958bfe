"""Benchmark: particle-steps/s of the multiphase SPH step on one GB300.

Workload ("plain method at scale, 3 phases"): 1,048,576 fluid particles on a
128 x 64 x 128 lattice (x, y, z; d = 0.005 m, h = 0.01 m) in a 1.28 x 0.64 x
0.64 m open box with two layers of boundary particles, volume fractions from 64
random spherical blobs (phases 1000 / 800 / 1.2 kg/m^3), linear EOS with
stiffness 3 Pa m^3/kg, dt = 1e-4 s, seeded synthetic data. (A 128^3 block at
d = 0.005 m would fill the 0.64 m height exactly, leaving no room for the
boundary layers, so the block is half as tall and the same 2^20 particles.)

A step is one fused pass of the whole pipeline (hash, stable counting sort,
reorder, density + EOS, force + drift velocity, volume-fraction advance +
correction + advection) replayed from a captured CUDA graph. The soft EOS lets
the fluid compress under gravity: neighbour counts grow from ~29 to ~90 per
particle over the 2000 timed steps, and the per-stage times used for the
roofline are averaged over the same trajectory (a second context replays it,
timing one eager step with CUDA events every `--profile-every` steps). `value` counts
fluid particles only (boundary particles are processed but not counted) and
the state stays resident in HBM; `e2e` is the same metric through the public
API with one upload of the reference records from pinned host memory and a
per-step download of the display records (the reference's per-frame
TransferFromCUDA, here asynchronous so each copy overlaps the next step),
timed on the host clock.

--impl reference times the reference's own algorithm on the host cores: the
CPU oracle (a statement-by-statement restatement of the reference kernels,
bit-identical to them) on the same scene, all host threads, the same metric.

--workload dam_break measures the 32^3 two-phase dam break (32,768 fluid
particles, d = 0.01 m, h = 0.02 m, 0.64 m box, gas sphere, linear EOS k = 3,
dt = 2e-4 s) on the GPU (captured graph, CUDA events) with the CPU oracle on the
same scene beside it; with --impl reference, the CPU oracle alone.

--workload batched measures the batched configuration instead (not the headline
line): 512 independent two-phase bubble scenes, particle counts log-uniform in
[4096, 65536], 1-4 gas bubbles of radius 3h-8h each, h = 0.02 m, tiled into one
domain so that every pass covers all scenes in one launch; particle-steps/s over
all scenes' fluid particles, device-resident, CUDA events on the launch stream.

--workload large_step measures whether one step of 8 dt can stand in for 8
plain steps (the premise of a learned large-step corrector): on a 262,144-particle
bubble scene (d = 0.005 m, h = 0.01 m, dt = 1e-4 s, linear EOS k = 3) with its gas
bubbles and with the same lattice all liquid, after 600 plain steps, 16 steps of
8 dt against 128 plain steps, particles matched by bornid: rms and max relative
density error and rms velocity error of the liquid, and the wall time of both.

--workload device_ref measures the 2^20-particle lattice with the reference's only
EOS (Tait) and liquid phases (1000 / 800 kg/m^3: Tait diverges next to the
1.2 kg/m^3 gas), plain SPH (RunSimpleSPH: sort, density, force, advance), in two
arms: this library (reference call order and fused, captured graphs), and with
--impl reference the reference's own GPU kernels (fluid_system_kern.cu built
unmodified for sm_103a, driven with the reference's launch sequence by
oracle/ref_gpu.py, checked against the oracle in tests/test_gpu_device_ref.py),
timed as its wrappers run (a host synchronisation after every call) and
stream-ordered. The reference arm needs oracle/_ref/sph_ref_kern.cubin (built
where the reference checkout exists).

--workload learned measures the learned large-step corrector: its training
throughput (Adam steps at 65,536-row minibatches on pairs from three 64 x 128 x
64 scenes of the rollout's physics) and the audited rollout (8 dt steps, a plain
audit every 16, 1 % tolerance) of the 256 x 128 x 128 lattice (d = 0.005 m,
h = 0.01 m, dt = 1e-4 s, linear EOS k = 3) against the plain pipeline over the
same simulated time, with 256 gas bubbles (value) and all liquid; host clock.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
       [--workload dam_break|batched|large_step|device_ref|learned]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "sph-multiphase_gb300"))
sys.path.insert(0, REPO)

METRIC = "particle-steps/s at 1M (1 GB300)"
UNIT = "particle-steps/s"
# algorithmic bytes per particle for each stage of a fused step (HBM, FP32 SoA;
# neighbour re-reads assumed to hit L2 / shared memory)
ALGO_BYTES = {"hash": 24, "cell_starts": 0, "cell_order": 16, "rearrange": 128, "density": 24,
              "force_drift": 136, "alpha_correct_advance": 168, "advance": 168}
# hash, 3 scan, scatter, cell sort, big-cell sort, rearrange (with the slot map), bucket density,
# list expansion, force + drift, alpha + correction + advance
KERNELS_PER_FUSED_STEP = 12


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Replicas:
    """Independent replicas, one per rank (the step has no data exchange): a
    barrier around the timed region and the maximum of the per-rank times."""

    def __init__(self, backend=None):
        self.ws, self.rank, self.local = _dist()
        self.dist = None
        if self.ws > 1:
            import torch
            import torch.distributed as dist
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist
            self.device = "cuda" if backend == "nccl" else "cpu"

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, value):
        if self.dist is None:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic(stage):
    """DRAM bytes per launch of `stage` from the committed ncu summary, if any."""
    try:
        with open(os.path.join(REPO, "profiles", "ncu_traffic.json")) as f:
            d = json.load(f)
        v = d.get(stage)
        return None if v is None else float(v)
    except Exception:
        return None


def _ncu_counts(stage):
    """Warp instructions per launch of `stage` (smsp__inst_executed.sum, summed over the
    stage's kernels) from the committed ncu summary, if any."""
    try:
        with open(os.path.join(REPO, "profiles", "ncu_counts.json")) as f:
            d = json.load(f)
        v = d.get("inst_per_launch", {}).get(stage)
        return None if v is None else float(v)
    except Exception:
        return None


SM_COUNT = 152
SCHEDULERS_PER_SM = 4


def roofline_line(dom, stages, samples, units, algo, achieved, peak, peak_kind, step_bytes, clocks):
    """The roofline object: the dominant stage against the measured HBM bandwidth, its DRAM
    traffic, and its issue-slot utilisation (warp instructions per launch from ncu over the
    scheduler slots of the timed launch at the sampled SM clock); `bound` names the limit
    the two fractions point to."""
    frac = achieved / peak
    traffic = _traffic(dom)
    step_dram = None
    try:
        with open(os.path.join(REPO, "profiles", "ncu_traffic.json")) as f:
            d = json.load(f)
        step_dram = sum(float(v) for k, v in d.items() if not k.startswith("_"))
    except Exception:
        pass
    issue = None
    inst = _ncu_counts(dom)
    mhz = clocks.get("sm_mhz") or 2070
    if inst is not None:
        slots = stages[dom] * 1e-3 * SM_COUNT * SCHEDULERS_PER_SM * mhz * 1e6
        issue = {"inst_per_launch": inst, "achieved_inst_per_s": inst / (stages[dom] * 1e-3),
                 "peak_inst_per_s": SM_COUNT * SCHEDULERS_PER_SM * mhz * 1e6, "frac": inst / slots,
                 "how": "smsp__inst_executed.sum per launch (profiles/ncu_counts.json) over 152 SMs x 4 "
                        "schedulers x the median SM clock sampled during the timed steps"}
    if frac >= 0.5:
        bound = "hbm"
    elif issue is not None and issue["frac"] >= 0.5:
        bound = "issue"
    else:
        bound = "latency"
    return {"bound": bound, "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": frac,
            "peak_source": peak_kind, "denominator": "measured HBM copy bandwidth (MEASURED_PEAKS.json)",
            "traffic": traffic, "algorithmic_bytes_per_launch": algo, "launch_ms": stages[dom],
            "launch_ms_from": f"mean of {samples} eager steps spread over the timed steps (CUDA events)",
            "issue": issue, "step_algorithmic_bytes": step_bytes, "step_dram_bytes": step_dram,
            "step_dram_from": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, summed over the "
                              "stages (profiles/ncu_traffic.json)"}


class ClockSampler:
    """nvidia-smi SM clocks / throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"sphmp_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9 and parts[1].isdigit():
                        rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [int(r[1]) for r in rows]
        mx = max(int(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


LATTICE = (128, 64, 128)


def build_scene(seed, gen=None, lattice=LATTICE):
    """The benchmark scene; `gen` = the scene generators (default: the library's; the reference
    arm passes the oracle's restatement, which builds the same records byte for byte without
    loading the CUDA library). A smaller `lattice` keeps the scene's physics and box (profiling
    captures that must stay small)."""
    from sphmp import abi, scenes
    return scenes.blobs_3phase(seed=seed, lattice=tuple(lattice), eos=abi.EOS_LINEAR, eos_k=3.0,
                               gen=gen or scenes.LIBRARY)


def scene_config(scene):
    """The workload description both arms print in `config` (identical for the same scene)."""
    p = scene.params
    return {"workload": scene.name, "fluid_particles": scene.n_fluid, "boundary_particles": scene.n_boundary,
            "phases": int(p.nphase), "h": 0.01, "d": 0.005, "box": [1.28, 0.64, 0.64], "dt": 1e-4,
            "eos": "linear k=3", "schedule": SCHEDULE_NAME, "seed": None}


SCHEDULE_NAME = "fused (3 neighbour passes)"


def cpu_sample(scene, steps, budget_s, threads=None, warmup=1):
    """Time the CPU oracle on the bench scene (the fused schedule, as the GPU arm) after `warmup`
    untimed steps (their own budget of budget_s); returns (particle-steps/s, steps done, seconds,
    threads, warm-up steps done)."""
    from oracle import oracle as O
    from sphmp import abi
    O.build()
    if threads:
        O.set_threads(threads)
    nthr = O.lib().orc_get_num_threads()
    p = scene.params
    s = O.state_from_aos(scene.disp, scene.calc, p.gridtotal)
    import numpy as np
    for k in range(p.nphase):
        s.alpha[:, k] = scene.calc["restdens"] == np.float32(p.densArr[k])
    s.alpha_pre[:] = s.alpha
    O.before_first_step(p, s)
    warm = 0
    tw = time.perf_counter()
    while warm < max(1, warmup):  # page-in, thread pool
        O.step(p, s, abi.SCHEDULE_FUSED, 1)
        warm += 1
        if time.perf_counter() - tw > budget_s:
            break
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        O.step(p, s, abi.SCHEDULE_FUSED, 1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return scene.n_fluid * done / dt, done, dt, nthr, warm


def _repo_libraries():
    """Shared libraries of this repository mapped into this process (Linux /proc/self/maps)."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so") and REPO in ln}
        return sorted(os.path.relpath(p, REPO) for p in paths)
    except OSError:
        return None


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from oracle import oracle as O
    scene = build_scene(args.seed, gen=O.Generators, lattice=args.lattice)  # the oracle's generators: no CUDA
    # warm-up steps are part of the sample's own warm-up; the timed part is bounded
    value, done, dt, nthr, warm = cpu_sample(scene, max(1, args.steps), budget_s=args.cpu_budget,
                                             warmup=args.warmup)
    cfg = scene_config(scene)
    cfg["seed"] = args.seed
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": done, "warmup": warm, "ms_per_step": 1000.0 * dt / max(done, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthr, "kind": "port",
                         "sample": f"{done} fused steps of the {scene.n_fluid}-fluid-particle scene on the oracle "
                                   f"(capped at {args.cpu_budget:.0f} s; requested {args.steps}); scene built by "
                                   f"the oracle's generators, no CUDA library loaded"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "repo_libraries_loaded": _repo_libraries(),
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    import sphmp
    from sphmp import abi

    rep = Replicas()
    ws, rank, local = rep.ws, rep.rank, rep.local
    torch.cuda.set_device(local)
    dev_index = torch.cuda.current_device()
    scene = build_scene(args.seed + rank, lattice=args.lattice)
    scene.params.cell_order = abi.CELL_ORDER_MORTON if args.cell_order == "morton" else abi.CELL_ORDER_LINEAR
    n_fluid = scene.n_fluid

    ctx = sphmp.Context(scene.params)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_aos(scene.disp, scene.calc)
    ctx.before_first_step()
    ctx.step(args.warmup, abi.SCHEDULE_FUSED, use_graph=True)   # includes graph capture
    ctx.sync()

    barrier = rep.barrier

    # ---- device-resident timed region ----
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev_index) as clk:
        ev0.record(stream)
        ctx.step(args.steps, abi.SCHEDULE_FUSED, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = rep.max(ev0.elapsed_time(ev1))
    ctx.sync()
    n_in = int((ctx.download_field(abi.F_MGCELL) != abi.GRID_UNDEF).sum())
    cons = ctx.conservation()

    ctx.close()

    # ---- per-stage times over the same trajectory (CUDA events on the launch stream) ----
    ctx = sphmp.Context(scene.params)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_aos(scene.disp, scene.calc)
    ctx.before_first_step()
    ctx.step(args.warmup, abi.SCHEDULE_FUSED, use_graph=True)
    stages = {}
    # at least five samples spread over the timed steps, at most one every --profile-every steps
    every = max(1, min(args.profile_every, args.steps // 5))
    samples = 0
    done = 0
    while done < args.steps:
        for name, t in ctx.step_profile(abi.SCHEDULE_FUSED):
            stages[name] = stages.get(name, 0.0) + t
        samples += 1
        seg = min(every, args.steps - done)
        if seg > 1:
            ctx.step(seg - 1, abi.SCHEDULE_FUSED, use_graph=True)
        done += seg
    stages = {k: v / samples for k, v in stages.items()}
    dom = max((k for k in stages if k in ALGO_BYTES and ALGO_BYTES[k] > 0), key=lambda k: stages[k])
    units = ctx.n
    algo = ALGO_BYTES[dom] * units
    achieved = algo / (stages[dom] * 1e-3) / 1e9
    peak, peak_kind = _peaks()
    step_bytes = sum(ALGO_BYTES.get(k, 0) for k in stages) * units
    ctx.close()

    # ---- end to end through the public API, host buffers ----
    e2e_steps = args.steps if args.e2e_steps <= 0 else max(1, min(args.steps, args.e2e_steps))
    pin_disp = torch.empty(scene.n * 32, dtype=torch.uint8, pin_memory=True)
    pin_calc = torch.empty(scene.n * 224, dtype=torch.uint8, pin_memory=True)
    pin_out = [torch.empty(scene.n * 32, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
    hd = pin_disp.numpy().view(abi.display_dtype())
    hc = pin_calc.numpy().view(abi.calc_dtype())
    ho = [t.numpy().view(abi.display_dtype()) for t in pin_out]
    hd[:] = scene.disp
    hc[:] = scene.calc
    ctx2 = sphmp.Context(scene.params)
    ctx2.set_stream(stream.cuda_stream)
    ctx2.upload_aos(hd, hc)
    ctx2.before_first_step()
    ctx2.step(args.warmup, abi.SCHEDULE_FUSED, use_graph=True)
    ctx2.download_aos(calc=False, out=(ho[0], None))
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx2.upload_aos(hd, hc)
    ctx2.before_first_step()
    for k in range(e2e_steps):
        ctx2.step(1, abi.SCHEDULE_FUSED, use_graph=True)
        ctx2.download_display_async(ho[k & 1])   # copy of step k overlaps step k + 1
    ctx2.download_wait()
    torch.cuda.synchronize()
    e2e_s = rep.max(time.perf_counter() - t0)
    ctx2.close()

    value = ws * n_fluid * args.steps / (ms * 1e-3)
    e2e_value = ws * n_fluid * e2e_steps / e2e_s
    clocks = clk.summary()
    cfg = scene_config(scene)
    cfg["seed"] = args.seed
    if args.cell_order != "linear":
        cfg["cell_order"] = args.cell_order
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "run": {"graph": True, "l2": "working set ~0.5 GB > 129 MB L2 (no flush needed)",
                "parallelism": f"replicas x{ws}", "in_grid_after": n_in,
                "stage_ms": {k: round(v, 4) for k, v in stages.items()},
                "stage_ms_from": f"mean of {samples} eager steps spread over the timed steps",
                "mass_fp64": cons["mass"], "alpha_sum_err": cons["alpha_sum_err"]},
        "roofline": roofline_line(dom, stages, samples, units, algo, achieved, peak, peak_kind, step_bytes,
                                  clocks),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": scene.n * 256 / e2e_steps,
                "d2h_bytes_per_step": scene.n * 32,
                "how": f"one TransferToCUDA upload + sort, then {e2e_steps} x (step + display download "
                       f"to pinned host memory, each copy overlapping the next step), host clock"},
        "gpu_launches": KERNELS_PER_FUSED_STEP * args.steps,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        v, done, dt, nthr, _ = cpu_sample(scene, args.cpu_steps, budget_s=args.cpu_budget)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nthr, "kind": "port",
                                "sample": f"{done} fused steps of the same scene on the CPU oracle "
                                          f"({dt:.1f} s, {nthr} threads)"}
    if rank == 0:
        print(json.dumps(line))
    rep.close()
    return 0


def build_batched(seed, nscenes=512):
    import numpy as np
    from sphmp import scenes
    rng = np.random.default_rng(seed)
    counts = np.floor(np.exp(rng.uniform(np.log(4096), np.log(65536), nscenes))).astype(int)
    parts = [scenes.bubble_scene(seed=seed * 100003 + i, n_particles=int(c)) for i, c in enumerate(counts)]
    big, _ = scenes.tile(parts)
    return big, nscenes


def run_batched(args):
    import torch

    import sphmp
    from sphmp import abi

    rep = Replicas()
    torch.cuda.set_device(rep.local)
    scene, nscenes = build_batched(args.seed + rep.rank)
    stream = torch.cuda.Stream()
    ctx = sphmp.Context(scene.params)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_aos(scene.disp, scene.calc)
    ctx.before_first_step()
    ctx.step(args.warmup, abi.SCHEDULE_FUSED, use_graph=True)
    ctx.sync()
    # the launch-shape autotuner on the warmed state (timed trials in a scratch context); the
    # hand-swept default is its first trial
    tuning = ctx.autotune(trial_steps=args.tune_steps, allow_reorder=args.cell_order == "morton") \
        if args.tune_steps > 0 else None
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    rep.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        ev0.record(stream)
        ctx.step(args.steps, abi.SCHEDULE_FUSED, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize()
    rep.barrier()
    ms = rep.max(ev0.elapsed_time(ev1))
    stages = {name: t for name, t in ctx.step_profile(abi.SCHEDULE_FUSED)}  # the state after the timed steps
    ctx.close()
    line = {
        "metric": "particle-steps/s, 512 batched scenes (1 GB300)", "value": rep.ws * scene.n_fluid * args.steps
        / (ms * 1e-3), "unit": UNIT, "n_gpus": rep.ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched_{nscenes}_bubble_scenes", "scenes": nscenes,
                   "fluid_particles": scene.n_fluid, "boundary_particles": scene.n_boundary, "h": 0.02,
                   "d": 0.01, "dt": 2e-4, "eos": "linear k=3", "schedule": "fused, one launch per pass for all "
                   "scenes (spatial tiling)", "graph": True, "stage_ms_after": {k: round(v, 4) for k, v in
                                                                                  stages.items()},
                   "autotune": tuning},
        "gpu_launches": KERNELS_PER_FUSED_STEP * args.steps,
        "clocks": clk.summary(),
    }
    if rep.rank == 0:
        print(json.dumps(line))
    rep.close()
    return 0


def run_large_step(args):
    import tempfile

    import numpy as np
    import torch

    import sphmp
    from sphmp import abi, scenes

    stream = torch.cuda.Stream()

    def state(ctx):
        d = {k: ctx.download_field(f) for k, f in (("dens", abi.F_DENS), ("vel", abi.F_VEL),
                                                    ("bornid", abi.F_BORNID), ("type", abi.F_TYPE),
                                                    ("restdens", abi.F_RESTDENS), ("mgcell", abi.F_MGCELL))}
        o = np.argsort(d["bornid"], kind="stable")
        return {k: v[o] for k, v in d.items()}

    def run(prm, path, nsteps):
        """nsteps eager steps from the saved state; CUDA-event milliseconds and the final state."""
        c = sphmp.Context(prm)
        c.set_stream(stream.cuda_stream)
        c.load_state(path)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        c.step(nsteps, abi.SCHEDULE_FUSED, use_graph=False)
        ev1.record(stream)
        torch.cuda.synchronize()
        st = state(c)
        c.close()
        return ev0.elapsed_time(ev1), st

    cases = {}
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "state.bin")
        for case in ("bubbles", "liquid"):
            sc = scenes.bubble_scene(seed=5, n_particles=262144, d=0.005, h=0.01, dt=1e-4)
            if case == "liquid":
                sc.calc["restdens"][:sc.n_fluid] = sc.params.densArr[0]
                sc.calc["mass"][:sc.n_fluid] = sc.params.massArr[0]
            p = sc.params
            ctx = sphmp.Context(p)
            ctx.set_stream(stream.cuda_stream)
            ctx.upload_aos(sc.disp[:sc.n], sc.calc[:sc.n])
            ctx.before_first_step()
            ctx.step(600, abi.SCHEDULE_FUSED, use_graph=True)
            ctx.save_state(path)
            vmax = float(np.sqrt((ctx.download_field(abi.F_VEL) ** 2).sum(1)).max())
            ctx.close()
            p8 = p.copy()
            p8.dt = p.dt * 8
            ms_plain, a = run(p, path, 128)
            ms_large, b = run(p8, path, 16)
            liq = ((a["type"] == 0) & (a["restdens"] > 500) & (a["mgcell"] != abi.GRID_UNDEF)
                   & (b["mgcell"] != abi.GRID_UNDEF))
            ra, rb = 1.0 / a["dens"][liq], 1.0 / b["dens"][liq]
            rel = (rb - ra) / ra
            va, vb = a["vel"][liq], b["vel"][liq]
            vrms = float(np.sqrt(np.mean(np.sum(va ** 2, 1))))
            cases[case] = {"liquid_particles": int(liq.sum()), "density_err_rms": float(np.sqrt(np.mean(rel ** 2))),
                           "density_err_max": float(np.abs(rel).max()),
                           "velocity_err_rms_over_rms": float(np.sqrt(np.mean(np.sum((vb - va) ** 2, 1)))) / vrms,
                           "velocity_rms": vrms, "max_speed_at_step_600": vmax,
                           "ms_128_plain_steps": ms_plain, "ms_16_large_steps": ms_large,
                           "sim_s_per_wall_s_ratio": ms_plain / ms_large}
    line = {"metric": "one 8 dt step against 8 plain steps (the premise of a learned large-step corrector)",
            "unit": "relative error", "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "bubbles_262144", "d": 0.005, "h": 0.01, "dt": 1e-4, "eos": "linear k=3",
                       "start": "after 600 plain steps", "compare": "16 steps of 8 dt against 128 plain steps, "
                       "liquid particles matched by bornid", "timing": "CUDA events, eager steps on both sides"},
            "cases": cases}
    print(json.dumps(line))
    return 0


def run_learned(args):
    """The learned corrector's configurations: training throughput at a
    65,536-particle minibatch, then the audited rollout on the 256 x 128 x 128
    lattice against the plain pipeline over the same simulated time."""
    import numpy as np
    import torch

    import sphmp
    from sphmp import abi, scenes
    from sphmp import learned as SL

    dev = torch.device("cuda", torch.cuda.current_device())
    torch.manual_seed(1)  # the timed Adam steps' minibatches: the same network in every run
    factor, audit_every, tol = 8, 16, 0.01
    sim_steps = args.learned_steps
    flop_per_sample = 3 * 2 * (48 * 128 + 2 * 128 * 128 + 128 * 4)  # forward + backward (2x forward)

    def fresh(sc, warm):
        c = sphmp.Context(sc.params)
        c.upload_aos(sc.disp[:sc.n], sc.calc[:sc.n])
        c.before_first_step()
        c.step(warm, abi.SCHEDULE_FUSED, use_graph=True)
        c.sync()
        return c

    cases, training = {}, {}
    for case in ("bubbles", "liquid"):
        liquid = case == "liquid"
        # training pairs from the batched plain solver: three scenes of the rollout's physics and
        # depth (64 x 128 x 64 sites, 32 bubbles: the rollout lattice's bubble density) tiled into
        # one domain, so that every pass of their plain steps covers all three in one launch; 16
        # starts spread over the rollout's time span, a quarter of each start's particles
        t0 = time.perf_counter()
        gen = torch.Generator(device=dev)
        gen.manual_seed(3)
        tiled, _ = scenes.tile([scenes.rollout_bubbles(seed=seed, lattice=(64, 128, 64), n_bubbles=32,
                                                       liquid_only=liquid) for seed in (21, 22, 23)])
        c = fresh(tiled, 50)
        large, plain = sphmp.Context(tiled.params), sphmp.Context(tiled.params)
        X, T = SL.generate_pairs(c, large, plain, factor, starts=16, gap=max(1, sim_steps // 16))
        keep = torch.randperm(X.shape[0], device=dev, generator=gen)[: X.shape[0] // 4]
        X = torch.nan_to_num(X[keep], nan=0.0, posinf=0.0, neginf=0.0)
        T = np.nan_to_num(T[keep.cpu().numpy()], nan=0.0, posinf=0.0, neginf=0.0)
        for x in (c, large, plain):
            x.close()
        t_pairs = time.perf_counter() - t0
        shift, scale, osc = SL.normalisation(X, T)
        cor = sphmp.Corrector(65536)
        cor.set_params(SL.init_params(0))
        cor.set_normalisation(shift, scale, osc)
        Tn = torch.from_numpy(T / osc).to(dev)
        SL.train(cor, X, Tn, 20, 65536, 1e-3, seed=1)  # warm-up
        batches = [torch.randint(0, X.shape[0], (65536,), device=dev) for _ in range(4)]
        xb = [X[i].contiguous() for i in batches]
        tb = [Tn[i].contiguous() for i in batches]
        nsteps = 400
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(nsteps):
            cor.train_step(xb[k % 4], tb[k % 4], 1e-3)
        e1.record()
        torch.cuda.synchronize()
        ms_train = e0.elapsed_time(e1) / nsteps
        log = SL.train(cor, X, Tn, 1500, 65536, 1e-3, seed=2, log_every=1499)
        training[case] = {"pairs": int(X.shape[0]), "pair_generation_s": round(t_pairs, 2), "batch": 65536,
                          "ms_per_adam_step": ms_train, "samples_per_s": 65536 / (ms_train * 1e-3),
                          "tflops": 65536 * flop_per_sample / (ms_train * 1e-3) / 1e12,
                          "loss_first_last": [log[0][1], log[-1][1]]}
        print(f"learned/{case}: trained on {X.shape[0]} pairs, {training[case]}", file=sys.stderr, flush=True)
        # rollout on the full lattice
        sc = scenes.rollout_bubbles(seed=9, liquid_only=liquid)
        src = fresh(sc, 50)
        res = {"fluid_particles": sc.n_fluid, "boundary_particles": sc.n_boundary}
        for arm in ("plain", "learned"):
            ctx = sphmp.Context(sc.params)
            aud = sphmp.Context(sc.params) if arm == "learned" else None
            if arm == "learned":  # one audited large step: the rollout's buffers are allocated
                ctx.copy_state_from(src)
                ctx.rollout(aud, factor, factor=factor, corrector=cor, audit_every=audit_every, tol=tol)
            ctx.copy_state_from(src)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if arm == "plain":
                ctx.step(sim_steps, abi.SCHEDULE_FUSED, use_graph=True)
                ctx.sync()
                st = None
            else:
                st = ctx.rollout(aud, sim_steps, factor=factor, corrector=cor, audit_every=audit_every, tol=tol)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            res[arm] = {"wall_s": wall, "sim_s_per_wall_s": sim_steps * sc.params.dt / wall}
            print(f"learned/{case}/{arm}: {res[arm]} {st}", file=sys.stderr, flush=True)
            if st:
                res[arm]["stats"] = st
            if arm == "plain":
                ref = ctx
            else:
                for c in (ctx, ref):
                    c.sort()
                    c.compute_pressure()
                res["learned_vs_plain_at_end"] = ctx.compare_to(ref)
                ctx.close()
                aud.close()
                ref.close()
        # references for the end-of-run difference: the plain pipeline from the start state moved
        # by one ulp in x (how far two faithful trajectories drift apart over the same time: the
        # floor under any method's error against the plain run) and, all liquid, the same audited
        # rollout without the network
        ref = sphmp.Context(sc.params)
        ref.copy_state_from(src)
        ref.step(sim_steps, abi.SCHEDULE_FUSED, use_graph=True)
        ref.sort()
        ref.compute_pressure()
        for arm in (("uncorrected", "plain_one_ulp") if liquid else ("plain_one_ulp",)):
            ctx = sphmp.Context(sc.params)
            ctx.copy_state_from(src)
            if arm == "uncorrected":
                aud = sphmp.Context(sc.params)
                st = ctx.rollout(aud, sim_steps, factor=factor, corrector=None, audit_every=audit_every, tol=tol)
                aud.close()
                res[arm] = {"stats": st}
            else:
                pos = ctx.download_field(abi.F_POS)
                pos[:, 0] = np.nextafter(pos[:, 0], np.float32(np.inf))
                ctx.upload_field(abi.F_POS, pos)
                ctx.step(sim_steps, abi.SCHEDULE_FUSED, use_graph=True)
                res[arm] = {}
            ctx.sort()
            ctx.compute_pressure()
            res[arm]["vs_plain_at_end"] = ctx.compare_to(ref)
            print(f"learned/{case}/{arm}: {res[arm]}", file=sys.stderr, flush=True)
            ctx.close()
        ref.close()
        res["sim_s_per_wall_s_ratio"] = res["learned"]["sim_s_per_wall_s"] / res["plain"]["sim_s_per_wall_s"]
        cases[case] = res
        src.close()
        cor.close()
    line = {"metric": "learned vs plain sim-s/wall-s at <=1% density and volume-fraction error",
            "value": cases["bubbles"]["sim_s_per_wall_s_ratio"], "unit": "x (sim-s/wall-s, learned over plain)",
            "n_gpus": 1, "higher_is_better": True, "dtype": "bf16 network (FP32 accumulate), f32 solver",
            "data": "synthetic",
            "config": {"workload": "rollout_256x128x128_2phase_256bubbles", "d": 0.005, "h": 0.01, "dt": 1e-4,
                       "large_step": f"{factor} dt", "audit_every_large_steps": audit_every, "tolerance": tol,
                       "simulated_s": sim_steps * 1e-4, "eos": "linear k=3",
                       "training": "pairs from the batched plain solver: 3 scenes of 64x128x64 sites with the "
                                   "rollout's physics and depth (32 bubbles each, or all liquid) tiled into one "
                                   "domain, 16 starts over the rollout's time span, a quarter of each start's "
                                   "particles; 1500 Adam steps at 65,536 per batch, lr 1e-3",
                       "timing": "host clock around each arm (the rollout synchronises at its audits)"},
            "cases": cases, "training": training}
    print(json.dumps(line))
    return 0


def device_ref_scene(seed):
    """The benchmark lattice with the reference's only EOS (Tait) and liquid phases:
    the 1.2 kg/m^3 gas blobs become phase-0 liquid (Tait diverges next to them)."""
    import numpy as np
    from sphmp import abi, scenes
    sc = scenes.blobs_3phase(seed=seed, eos=abi.EOS_TAIT, multiphase=0)
    gas = sc.calc["restdens"][:sc.n] == np.float32(sc.params.densArr[2])
    sc.calc["restdens"][:sc.n][gas] = sc.params.densArr[0]
    sc.calc["mass"][:sc.n][gas] = sc.params.massArr[0]
    calc = sc.calc[:sc.n].copy()
    bnd = sc.disp["type"][:sc.n] == abi.TYPE_BOUNDARY
    calc["accel"][bnd] = 0  # as the oracle state starts
    calc["pressure"][bnd] = 0
    return sc, np.ascontiguousarray(sc.disp[:sc.n]), calc


DEVICE_REF_METRIC = "particle-steps/s at 1M, Tait liquid lattice, plain SPH (1 GB300)"


def device_ref_config(sc, what):
    return {"workload": "blobs_128x64x128_liquid_tait", "fluid_particles": sc.n_fluid,
            "boundary_particles": sc.n_boundary, "eos": "Tait (the reference's)", "phases": "1000 / 800 kg/m^3 blobs",
            "step": "plain SPH (RunSimpleSPH: sort, density + pressure, force, advance)", "timed": what}


def _timed(stream, fn):
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    fn()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


def run_device_ref_library(args):
    """This library on the device-ref scene (the sphmp arm of --workload device_ref)."""
    import numpy as np
    import torch

    import sphmp
    from sphmp import abi

    sc, disp, calc = device_ref_scene(args.seed)
    K, W = args.steps, args.warmup
    stream = torch.cuda.Stream()
    res = {}
    with ClockSampler(torch.cuda.current_device()) as clk:
        ctx = sphmp.Context(sc.params)
        ctx.set_stream(stream.cuda_stream)
        ctx.upload_aos(disp, calc)
        ctx.before_first_step()
        for name, sched in (("reference_order", abi.SCHEDULE_REFERENCE), ("fused", abi.SCHEDULE_FUSED)):
            ctx.step(W, sched, use_graph=True)
            res[name] = _timed(stream, lambda: ctx.step(K, sched, use_graph=True))
        ctx.sync()
        finite = bool(np.isfinite(ctx.download_field(abi.F_POS)).all())
        ctx.close()
    nf = sc.n_fluid
    line = {"metric": DEVICE_REF_METRIC, "value": nf * K / (res["reference_order"] * 1e-3), "unit": UNIT,
            "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": res["reference_order"] / K,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": device_ref_config(sc, "reference call order, captured graph (value); fused schedule (fused)"),
            "fused": {"value": nf * K / (res["fused"] * 1e-3), "ms_per_step": res["fused"] / K},
            "finite": finite, "gpu_launches": KERNELS_PER_FUSED_STEP * K,  # the reference-order step: 13 kernels too
            "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


def run_device_ref_reference(args):
    """The reference's own GPU kernels on the device-ref scene (the reference arm of
    --workload device_ref): fluid_system_kern.cu built for sm_103a, driven by
    oracle/ref_gpu.py with the reference's launch sequence."""
    import numpy as np
    import torch

    from oracle import ref_gpu
    from sphmp import abi

    if not ref_gpu.available():
        print(json.dumps({"impl": "reference", "workload": "device_ref",
                          "unavailable": "oracle/_ref/sph_ref_kern.cubin not built (needs the reference checkout "
                                         "at build time)"}))
        return 0
    sc, disp, calc = device_ref_scene(args.seed)
    K, W = args.steps, args.warmup
    stream = torch.cuda.Stream()
    with ClockSampler(torch.cuda.current_device()) as clk:
        R = ref_gpu.RefGPU(sc.params, disp, calc, stream=stream)
        R.before_first_step()
        R.step(W)
        R.sync_each = True
        ms = _timed(stream, lambda: R.step(K))
        R.sync_each = False
        R.step(W)
        ms_async = _timed(stream, lambda: R.step(K))
        d, _ = R.records(abi.display_dtype(), abi.calc_dtype())
        finite = bool(np.isfinite(d["pos"]).all())
        R.close()
    nf = sc.n_fluid
    line = {"metric": DEVICE_REF_METRIC, "value": nf * K / (ms * 1e-3), "unit": UNIT, "impl": "reference",
            "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic",
            "config": device_ref_config(sc, "the reference's kernels with a host synchronisation after every call, "
                                            "as its wrappers (value); stream-ordered (stream_ordered); "
                                            "thrust::sort_by_key replaced by the same stable key sort (torch.sort)"),
            "stream_ordered": {"value": nf * K / (ms_async * 1e-3), "ms_per_step": ms_async / K},
            "finite": finite, "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


def dam_break_scene(seed, gen=None):
    """The 32^3 two-phase dam break (32,768 fluid particles, d = 0.01 m, h = 0.02 m, 0.64 m
    box, gas sphere r = 0.06 m, linear EOS k = 3, dt = 2e-4 s)."""
    from sphmp import scenes
    return scenes.dam_break_2phase(seed=seed, n_side=32, gen=gen or scenes.LIBRARY)


def dam_break_config(sc, seed):
    return {"workload": sc.name, "fluid_particles": sc.n_fluid, "boundary_particles": sc.n_boundary, "phases": 2,
            "h": 0.02, "d": 0.01, "box": [0.64, 0.64, 0.64], "dt": 2e-4, "eos": "linear k=3",
            "schedule": SCHEDULE_NAME, "seed": seed}


def run_dam_break(args):
    """The dam break on the GPU (captured-graph steps, CUDA events on the launch stream) and the
    CPU oracle on the same scene (a bounded sample of the same steps)."""
    import torch

    import sphmp
    from sphmp import abi

    rep = Replicas()
    torch.cuda.set_device(rep.local)
    sc = dam_break_scene(args.seed + rep.rank)
    stream = torch.cuda.Stream()
    ctx = sphmp.Context(sc.params)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_aos(sc.disp, sc.calc)
    ctx.before_first_step()
    ctx.step(args.warmup, abi.SCHEDULE_FUSED, use_graph=True)
    ctx.sync()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    rep.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        ev0.record(stream)
        ctx.step(args.steps, abi.SCHEDULE_FUSED, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize()
    rep.barrier()
    ms = rep.max(ev0.elapsed_time(ev1))
    ctx.close()
    line = {
        "metric": "particle-steps/s, 32^3 two-phase dam break (1 GB300)",
        "value": rep.ws * sc.n_fluid * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": rep.ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dam_break_config(sc, args.seed + rep.rank),
        "run": {"graph": True, "l2": "working set ~20 MB, inside the 129 MB L2 (state resident, no flush)"},
        "gpu_launches": KERNELS_PER_FUSED_STEP * args.steps, "clocks": clk.summary(),
    }
    if rep.rank == 0 and not args.no_cpu_baseline:
        v, done, dt, nthr, _ = cpu_sample(sc, args.cpu_steps_dam, budget_s=args.cpu_budget)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nthr, "kind": "port",
                                "sample": f"{done} fused steps of the same scene on the CPU oracle "
                                          f"({dt:.1f} s, {nthr} threads)"}
    if rep.rank == 0:
        print(json.dumps(line))
    rep.close()
    return 0


def run_dam_break_reference(args):
    """--impl reference --workload dam_break: the CPU oracle alone on the dam break."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from oracle import oracle as O
    sc = dam_break_scene(args.seed, gen=O.Generators)
    value, done, dt, nthr, warm = cpu_sample(sc, max(1, args.steps), budget_s=args.cpu_budget, warmup=args.warmup)
    line = {
        "metric": "particle-steps/s, 32^3 two-phase dam break (1 GB300)", "value": value, "unit": UNIT,
        "impl": "reference", "n_gpus": args.gpus, "steps": done, "warmup": warm,
        "ms_per_step": 1000.0 * dt / max(done, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": dam_break_config(sc, args.seed),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthr, "kind": "port",
                         "sample": f"{done} fused steps of the dam break on the oracle (capped at "
                                   f"{args.cpu_budget:.0f} s; requested {args.steps})"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "repo_libraries_loaded": _repo_libraries(),
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="sphmp", choices=["sphmp", "reference"])
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end run (0: same as --steps)")
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--cpu-budget", type=float, default=30.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-every", type=int, default=100, help="steps between per-stage timing samples")
    ap.add_argument("--learned-steps", type=int, default=1280,
                    help="simulated time of the learned workload's rollout, in plain steps of dt")
    ap.add_argument("--lattice", default="128,64,128", type=lambda v: tuple(int(x) for x in v.split(",")),
                    help="blobs workload: fluid lattice x,y,z (the headline scene is 128,64,128; smaller ones are "
                         "for small profiling captures)")
    ap.add_argument("--cell-order", default="linear", choices=["linear", "morton"],
                    help="order of the cells in the sorted arrays (blobs workload): the reference's linear key "
                         "order (bit-exact sort, the default) or Z-order")
    ap.add_argument("--tune-steps", type=int, default=10,
                    help="batched workload: fused steps per autotuner trial (0: no autotuning)")
    ap.add_argument("--cpu-steps-dam", type=int, default=200, help="CPU-oracle sample of the dam-break workload")
    ap.add_argument("--workload", default="blobs",
                    choices=["blobs", "dam_break", "batched", "large_step", "device_ref", "learned"],
                    help="blobs: the headline 2^20-particle scene; dam_break: the 32^3 two-phase dam break "
                         "(GPU and CPU oracle); batched: 512 tiled bubble scenes; "
                         "large_step: one 8 dt step against 8 plain steps; device_ref: the Tait liquid lattice "
                         "(with --impl reference: the reference's own GPU kernels); learned: corrector training "
                         "and the audited rollout of the 256x128x128 bubble lattice against the plain pipeline")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "device_ref":
        return run_device_ref_reference(args) if args.impl == "reference" else run_device_ref_library(args)
    if args.workload == "dam_break":
        return run_dam_break_reference(args) if args.impl == "reference" else run_dam_break(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "large_step":
        return run_large_step(args)
    if args.workload == "learned":
        return run_learned(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
