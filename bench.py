"""Benchmark of the adaptive-grid simulation step on GB300.

Metric: active (leaf) cell-steps per second.

Workloads (--workload):
  batch (default) — 16 independent smoke plumes stepped as one batch: domain
    edges drawn (seed 0) from {64, 96, 128, 192, 256}, 2 or 3 levels, uneven
    block budgets, a sphere source in the bottom quarter of radius U[4,10] and
    temperature U[5,15], buoyancy, field-driven refinement, 100 Jacobi sweeps
    per level, and a seeded 16^3 emission map per member that the host uploads
    every step. The timed path is the mixed-precision batch (FP16 scalar
    storage, FP32 compute) with autotuned tiles and solve schedule, the whole
    step one CUDA graph. On the same plumes the line also reports the plain
    FP32 path (16 standalone simulations stepped one after another, each its
    own step graph), the FP32 batch, and the density error of FP16 storage
    against the FP64 oracle.
  cloud — one 3-level cloud scene at effective 256^3, 40k-block budget,
    terrain, wind inflow, temperature/vapor/density, field-driven
    refinement, 100 sweeps per level, FP32.
  large — the 512^3 4-level fire plume with a 100 GB block budget: FP16
    storage, FP32, and the uniform grid at the largest cube that fits 100 GB
    (no CPU baseline or end-to-end leg at this size).
  precision — not a timing: the cloud scene over 200 steps in FP32, FP16 and
    BF16 scalar storage, per-field relative L2 error against the FP64 oracle
    from 10 to 200 steps.

Synthetic inputs throughout (seeded sources, terrain, noise, emission maps);
scenes are spun up untimed before warm-up so the refined topology has
developed.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--workload batch|cloud|large|precision]
Under torchrun with N > 1 every rank runs an independent replica of the
workload (no data exchange); value sums the ranks' cell-steps over the
slowest rank's time.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ITERS = 100
CLOUD_SPINUP = 60
BATCH_N = 16
BATCH_SPINUP = 30
EM_N = 16
METRIC = "active cell-steps/s"


def batch_params(precision):
    from dcgrid_gb300 import scenes
    return scenes.plume_batch(BATCH_N, 0, sizes=(64, 96, 128, 192, 256), iters=ITERS, precision=precision,
                              em_n=EM_N)


def member_emission(i):
    from dcgrid_gb300 import scenes
    return scenes.emission_field(EM_N, 100 + i)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(name):
    """dram bytes per launch of a kernel from a committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            return json.load(f)
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, gpu_index=0):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or parts[0] != str(gpu_index):
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def reduce_max_sum(dist, torch, ms, cells, device):
    """Whole-job figures of N replicas: the slowest rank's time and the cells
    of all ranks (every rank receives both)."""
    a = torch.tensor([ms, float(cells)], dtype=torch.float64, device=device)
    dist.all_reduce(a[:1], op=dist.ReduceOp.MAX)
    dist.all_reduce(a[1:], op=dist.ReduceOp.SUM)
    return float(a[0].item()), float(a[1].item())


class Ctx:
    """Process / rank context: torch device, stream, optional process group."""

    def __init__(self):
        import torch
        self.torch = torch
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(self.local)
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            self.dist = dist
        from dcgrid_gb300 import build
        build.build()
        self.stream = torch.cuda.Stream()
        self.flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        # the clock samples of the timed region (DCG_CLOCKS_DIR, else the temp directory)
        import tempfile
        d = os.environ.get("DCG_CLOCKS_DIR") or tempfile.gettempdir()
        self.clock_path = os.path.join(d, f"dcg_clocks_r{self.rank}.csv")

    def barrier(self):
        if self.dist:
            self.dist.barrier()
        self.torch.cuda.synchronize()

    def max_sum(self, ms, cells):
        """max of the time and sum of the cells over the ranks"""
        if not self.dist:
            return ms, cells
        return reduce_max_sum(self.dist, self.torch, ms, cells, "cuda")

    def timed(self, steps, step_fn, cells_fn, nvtx="timed"):
        """device time of `steps` calls of step_fn (CUDA events on the sims'
        stream, L2 flushed before each step) and the active cells they covered"""
        torch = self.torch
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        cells = 0
        self.barrier()
        torch.cuda.nvtx.range_push(nvtx)  # lets ncu select the timed launches (--nvtx-include)
        for k in range(steps):
            with torch.cuda.stream(self.stream):
                self.flush.fill_(float(k))
            ev[k][0].record(self.stream)
            step_fn()
            ev[k][1].record(self.stream)
            cells += cells_fn()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        return sum(a.elapsed_time(b) for a, b in ev), cells

    def close(self):
        if self.dist:
            self.dist.barrier()
            self.dist.destroy_process_group()


def oracle_from_gpu(sim, p):
    """An FP64 oracle simulation holding the GPU simulation's topology and fields."""
    from oracle import pyoracle
    o = pyoracle.OracleSim(p, precision="double")
    if p.emission_n > 0:
        o.set_emission(sim._em)
    o.set_topology(sim.get_topology())
    names = ["density", "vel_x", "vel_y", "vel_z", "fluidity"]
    if p.n_scalars == 3:
        names += ["temperature", "vapor"]
    for f in names:
        o.set_field(f, sim.get_field(f).astype("float64"))
    return o


def cpu_sample(sims, params, steps=1):
    """The FP64 oracle on the host cores, started from the GPU states: `steps`
    steps of every simulation on all host threads, then the next `steps` steps
    of the same simulations on one thread; active cell-steps per second."""
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    orcs = [oracle_from_gpu(s, p) for s, p in zip(sims, params)]

    def rate(n_threads):
        pyoracle.set_threads(n_threads)
        cells = 0
        t0 = time.perf_counter()
        for o in orcs:
            for _ in range(steps):
                o.step(1)
                cells += o.stats().active_cells
        return cells / (time.perf_counter() - t0)

    value = rate(threads)
    one = rate(1)
    pyoracle.set_threads(threads)
    return {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} step(s) of each of the {len(sims)} simulation(s) from the GPU's spun-up state "
                      f"(same topology and fields), FP64 oracle, {threads} OpenMP threads",
            "single_core": {"value": one, "unit": METRIC, "cores": 1,
                            "sample": f"the next {steps} step(s) of the same simulations on one thread"}}


def density_error_fp16(params, steps=10):
    """Relative L2 density error of FP16 scalar storage against the FP64
    oracle after `steps` steps of the largest plume (both driven with the
    GPU's adaptation decisions so they share one topology)."""
    from dcgrid_gb300 import Simulation, capi
    from oracle import pyoracle
    import numpy as np
    i = max(range(len(params)), key=lambda k: params[k].max_blocks)
    p = params[i]
    q = capi.params_from_dict(capi.params_to_dict(p))
    q.precision = capi.PRECISION_MIXED_FP16
    g = Simulation(q)
    o = pyoracle.OracleSim(p, precision="double")
    em = member_emission(i)
    g.set_emission(em)
    o.set_emission(em)
    for s in (g, o):
        s.add_velocity_noise(0, 0.01)
    for _ in range(steps):
        g.advect_velocity()
        o.advect_velocity()
        g.adapt()
        mv, rf = g.get_last_adapt()
        o.adapt_replay(mv, rf)
        g.project()
        o.project()
        g.advect_scalars()
        o.advect_scalars()
    g.sync()
    alloc = np.repeat(o.get_topology()["pos"][:, 3] >= 0, 64)
    out = {"member": i, "domain": p.gx, "levels": p.levels, "steps": steps}
    for f in ["density", "temperature", "vel_y", "pressure"]:
        a = g.get_field(f)[alloc].astype(np.float64)
        b = o.get_field(f)[alloc]
        out[f] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
    g.close()
    return out


def reference_gpu_comparator(steps=3):
    """The reference's own kernels, compiled from its unmodified sources into
    oracle/_ref (cubins; the reference's host orchestration restated around
    them), against this library stage by stage on the same input: the
    reference's default scene at 64x128x64 (3000 blocks) and 256^3 (40000
    blocks), derived level counts, 10 (the reference's) and 100 Jacobi sweeps
    per level. A measurement of the reference, never a path of this library."""
    cubin = os.path.join(ROOT, "oracle", "_ref", "ref_dcgrid.cubin")
    if not os.path.exists(cubin):
        return {"unavailable": "the reference's cubins are not built (its sources were absent when build() ran)"}
    from oracle import ref_gpu_timing
    runs = []
    for size, blocks in [((64, 128, 64), 3000), ((256, 256, 256), 40000)]:
        for sweeps in (10, 100):
            runs.append(ref_gpu_timing.stage_compare(size, blocks, sweeps, steps=steps))
    return {"runs": runs,
            "note": "per stage: CUDA events on each side's stream after an L2 flush, mean of "
                    f"{steps} steps; ratio = reference ms / ours ms; adaptTopology on the reference side "
                    "includes its host ranking (D2H, sort, H2D) as in the reference application"}


# ------------------------------------------------------------------ batch
def run_batch(args, ctx):
    import numpy as np
    from dcgrid_gb300 import Batch, Simulation, capi
    torch = ctx.torch
    ems = [member_emission(i) for i in range(BATCH_N)]

    def make_batch(prec, defect_passes=0, tuning=None):
        params = batch_params(prec)
        for q in params:
            q.defect_passes = defect_passes
        b = Batch(params)
        b.set_stream(ctx.stream.cuda_stream)
        if tuning or args.tuning:  # a given schedule (profiling runs), else autotuned
            b.set_tuning(capi.tuning_from_dict(tuning or json.loads(args.tuning)))
            tune = capi.tuning_to_dict(b.get_tuning())
        else:
            tune = b.autotune(spinup_steps=5, reps=3)  # leaves the batch reset
        for i, m in enumerate(b):
            m.set_emission(ems[i])
            m._em = ems[i]
            m.add_velocity_noise(0, 0.01)
        b.step(BATCH_SPINUP + max(args.warmup, 3))
        b.sync()
        return b, tune

    def batch_cells(b):
        sts = b.stats()  # raises on a non-finite value (DCG_E_NAN)
        bad = [i for i, st in enumerate(sts) if st.device_error]
        if bad:
            raise RuntimeError(f"device error word set for members {bad}: "
                               f"{[hex(sts[i].device_error) for i in bad]}")
        return sum(st.active_cells for st in sts)

    # mixed-precision batch: the headline
    bm, tune_m = make_batch(capi.PRECISION_MIXED_FP16)
    clocks = Clocks(ctx.clock_path)
    clocks.start()
    ms, cells = ctx.timed(args.steps, lambda: bm.step(1), lambda: batch_cells(bm))
    clk = clocks.stop(ctx.local)
    bm.sync()  # raises when a device error word (timeout, budget, lookup, NaN) was set
    ms, cells = ctx.max_sum(ms, cells)
    value = cells / (ms * 1e-3)
    info = bm.info()
    if args.profile:  # the headline leg only (profiling runs)
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ctx.world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
                "config": {"workload": "profile: headline leg only", "tuning": tune_m},
                "gpu_launches": int(info["launches_per_step"] * args.steps)}
        bm.close()
        return line

    # FP32 batch (batching alone)
    bf, tune_f = make_batch(capi.PRECISION_FP32)
    ms_f, cells_f = ctx.timed(args.steps, lambda: bf.step(1), lambda: batch_cells(bf), "timed_fp32_batch")
    bf.sync()
    ms_f, cells_f = ctx.max_sum(ms_f, cells_f)
    batched_fp32 = cells_f / (ms_f * 1e-3)
    bf.close()

    # the mixed batch with one FP64 defect-correction pass after the cascade
    # (FP64 residual and norms, the FP32 cascade on the residual, p += e), on
    # the headline's schedule
    bd, _ = make_batch(capi.PRECISION_MIXED_FP16, defect_passes=1, tuning=tune_m)
    ms_d, cells_d = ctx.timed(args.steps, lambda: bd.step(1), lambda: batch_cells(bd), "timed_defect")
    bd.sync()
    ms_d, cells_d = ctx.max_sum(ms_d, cells_d)
    rel = [tuple(st.defect_rel_residual) for st in bd.stats()]
    defect = {"value": cells_d / (ms_d * 1e-3), "ms_per_step": ms_d / args.steps, "passes": 1,
              "cost_ms_per_step": (ms_d - ms) / args.steps,
              "rel_residual_before": max(r[0] for r in rel), "rel_residual_after": max(r[1] for r in rel),
              "rel_residual_note": "FP64 ||div - A p|| / ||div|| over every level's equations, worst member, "
                                   "before the first and after the last pass"}
    bd.close()

    # plain FP32 path: 16 standalone simulations, one after another on one stream
    plain = []
    for i, p in enumerate(batch_params(capi.PRECISION_FP32)):
        s = Simulation(p)
        s.set_stream(ctx.stream.cuda_stream)
        s.set_emission(ems[i])
        s.add_velocity_noise(0, 0.01)
        s.step(BATCH_SPINUP + max(args.warmup, 3))
        plain.append(s)
    for s in plain:
        s.sync()

    def plain_step():
        for s in plain:
            s.step(1)

    def plain_cells():
        sts = [s.stats() for s in plain]
        if any(st.device_error for st in sts):
            raise RuntimeError("device error word set in a plain FP32 simulation")
        return sum(st.active_cells for st in sts)

    ms_p, cells_p = ctx.timed(args.steps, plain_step, plain_cells, "timed_plain_fp32")
    for s in plain:
        s.sync()
    ms_p, cells_p = ctx.max_sum(ms_p, cells_p)
    plain_fp32 = cells_p / (ms_p * 1e-3)
    plain_launches = sum(s.launches_per_step() for s in plain)
    for s in plain:
        s.close()

    # end to end through the public API: per step the host uploads every
    # member's emission map (pinned host -> device), steps the batch, and reads
    # every member's statistics (mass, residual, active cells) back
    host_em = torch.from_numpy(np.concatenate([e.ravel() for e in ems])).pin_memory()
    ctx.barrier()
    t0 = time.perf_counter()
    e2e_cells = 0
    for k in range(args.steps):
        bm.set_emission(host_em)  # every member's map, one copy
        bm.step(1)
        e2e_cells += batch_cells(bm)
    torch.cuda.synchronize()
    e2e_ms, e2e_cells = ctx.max_sum((time.perf_counter() - t0) * 1e3, e2e_cells)
    bm.sync()
    stats_bytes = C.sizeof(capi.DcgStats)
    e2e = {"value": e2e_cells / (e2e_ms * 1e-3), "unit": METRIC,
           "h2d_bytes_per_step": 4 * EM_N ** 3 * BATCH_N, "d2h_bytes_per_step": stats_bytes * BATCH_N,
           "note": "per step: dcg_batch_set_emission (every member's map, one copy from pinned host memory), "
                   "dcg_batch_step, dcg_batch_get_stats (every member's statistics); host clock"}

    # roofline of the dominant kernel: the batched cooperative cascade
    peak, peak_kind = peaks()
    solve_ms, solve_bytes = bm.time_solve(5)
    achieved = solve_bytes / (solve_ms * 1e-3) / 1e9
    tr = committed_traffic("level_solve_batch_traffic.json")
    traffic = None
    if tr and tr.get("bytes_per_cell_sweep"):
        traffic = tr["bytes_per_cell_sweep"] * solve_bytes / 12.0
    roofline = {"bound": "hbm", "kernel": f"k_level_solve_batch (whole cascade: every round, {ITERS} sweeps each)",
                "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes_per_cascade": solve_bytes,
                "cascade_ms": solve_ms,
                "note": "algorithmic bytes: 12 per allocated cell per sweep (p read, div read, p~ write); "
                        "traffic: ncu dram bytes per cell-sweep of a smaller capture scaled to these cells; "
                        "the cascade is timed back to back (L2 warm between repetitions), the steps with "
                        "L2 flushed"}
    # the whole step against the per-cell-step byte count of the path:
    # 104 + (2k + 2) s_q + 12 N bytes per active cell-step (k scalars of s_q
    # bytes, N sweeps per level)
    kq = batch_params(0)[0].n_scalars
    step_bytes = 104 + (2 * kq + 2) * 2 + 12 * ITERS
    roofline["step_level"] = {"bytes_per_active_cell_step": step_bytes, "achieved": step_bytes * value / 1e9,
                              "frac": step_bytes * value / 1e9 / peak, "unit": "GB/s",
                              "note": f"k={kq} FP16 scalars (s_q=2), N={ITERS}: whole-step rate x bytes per "
                                      "active cell-step, against the same peak"}

    members = [{"edge": p.gx, "levels": p.levels, "max_blocks": p.max_blocks} for p in batch_params(0)]
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ctx.world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp16 storage / fp32 compute",
            "data": "synthetic (seeded plume sources, emission maps, velocity noise)",
            "config": {"workload": f"batch of {BATCH_N} independent plumes, edges from {{64,96,128,192,256}} "
                                   f"(seed 0), 2-3 levels, {ITERS} Jacobi sweeps/level, FP16 scalar storage / "
                                   f"FP32 compute, autotuned, one CUDA graph per step",
                       "members": members, "block_edge": 4, "spinup_steps": BATCH_SPINUP,
                       "emission": f"{EM_N}^3 map per member over the bottom 16 cell layers",
                       "tuning": tune_m, "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"replicas x{ctx.world}" if ctx.world > 1 else "single",
                       "active_cells_last_step": int(batch_cells(bm))},
            "comparison": {"plain_fp32_standalone": plain_fp32, "plain_fp32_ms_per_step": ms_p / args.steps,
                           "plain_fp32_launches_per_step": plain_launches,
                           "batched_fp32": batched_fp32, "batched_fp32_tuning": tune_f,
                           "speedup_vs_plain_fp32": value / plain_fp32,
                           "mixed_batch_fp64_defect_correction": defect,
                           "speedup_batching_fp32": batched_fp32 / plain_fp32},
            "gpu_launches": int(info["launches_per_step"] * args.steps),
            "launches_per_step": info["launches_per_step"], "roofline": roofline, "e2e": e2e}
    if clk:
        line["clocks"] = clk
    if ctx.rank == 0 and not args.no_ref_gpu:
        line["comparison"]["reference_gpu"] = reference_gpu_comparator()
    if ctx.rank == 0 and not args.no_cpu:
        # the largest member over the headline's horizon: spin-up, warm-up and timed steps
        line["comparison"]["rel_err_fp16_vs_fp64"] = density_error_fp16(
            batch_params(capi.PRECISION_FP32), BATCH_SPINUP + max(args.warmup, 3) + args.steps)
        line["cpu_baseline"] = cpu_sample(list(bm), batch_params(capi.PRECISION_FP32), 1)
    bm.close()
    return line


# ------------------------------------------------------------------ cloud
def run_cloud(args, ctx):
    from dcgrid_gb300 import Simulation, capi, scenes
    torch = ctx.torch
    p = scenes.cloud256()
    sim = Simulation(p)
    sim.set_stream(ctx.stream.cuda_stream)
    em = scenes.emission_field(EM_N, 1)
    sim._em = em
    sim.set_emission(em)
    sim.add_velocity_noise(0, 0.01)
    sim.step(CLOUD_SPINUP + max(args.warmup, 3))
    sim.sync()
    clocks = Clocks(ctx.clock_path)
    clocks.start()
    ms, cells = ctx.timed(args.steps, lambda: sim.step(1), lambda: sim.stats().active_cells)
    clk = clocks.stop(ctx.local)
    sim.sync()  # raises when the device error word was set
    ms, cells = ctx.max_sum(ms, cells)
    value = cells / (ms * 1e-3)
    launches = sim.launches_per_step()

    # end to end: per step upload the emission map (pinned host -> device) and
    # read back the dense density volume (device -> pinned host)
    g = p.gx
    host_out = torch.empty(g * g * g, dtype=torch.float32).pin_memory()
    host_em = torch.from_numpy(em).pin_memory()
    ctx.barrier()
    e2e_cells = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        sim.set_emission(host_em)
        sim.step(1)
        if sim.L.dcg_get_dense(sim.h, capi.FIELD_DENSITY, C.c_void_p(host_out.data_ptr()), capi.HOST):
            raise RuntimeError("dcg_get_dense failed")
        e2e_cells += sim.stats().active_cells
    torch.cuda.synchronize()
    e2e_ms, e2e_cells = ctx.max_sum((time.perf_counter() - t0) * 1e3, e2e_cells)
    e2e = {"value": e2e_cells / (e2e_ms * 1e-3), "unit": METRIC,
           "h2d_bytes_per_step": 4 * EM_N ** 3, "d2h_bytes_per_step": 4 * g * g * g,
           "note": "per step: dcg_set_emission from pinned host memory, dcg_step, dcg_get_dense into pinned "
                   "host memory, dcg_get_stats; host clock"}

    peak, peak_kind = peaks()
    jac_ms, jac_bytes = sim.time_kernel(4, 0, 5)
    achieved = jac_bytes / (jac_ms * 1e-3) / 1e9
    tr = committed_traffic("level_solve_cloud256_traffic.json")
    traffic = None
    if tr and tr.get("bytes_per_cell_sweep"):
        traffic = tr["bytes_per_cell_sweep"] * jac_bytes / 12.0
    roofline = {"bound": "hbm", "kernel": f"k_level_solve_batch (one member, level 0, {ITERS} sweeps per launch)",
                "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "algorithmic_bytes_per_launch": jac_bytes, "launch_ms": jac_ms,
                "note": "working set (p, p~, div of the level) is L2-resident across sweeps; frac > 1 "
                        "would mean L2 reuse beyond the HBM roofline"}
    st = sim.stats()
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ctx.world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded terrain, source bubble, emission map, velocity noise)",
            "config": {"workload": f"adaptive cloud scene, effective 256^3, 3 levels, 40000 block budget, "
                                   f"{ITERS} Jacobi sweeps/level",
                       "domain": [g, g, g], "levels": 3, "max_blocks": 40000, "jacobi_iters": ITERS,
                       "block_edge": 4, "spinup_steps": CLOUD_SPINUP, "n_scalars": 3,
                       "emission": f"{EM_N}^3 map over the bottom 16 cell layers",
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"replicas x{ctx.world}" if ctx.world > 1 else "single",
                       "active_cells_last_step": int(st.active_cells)},
            "gpu_launches": int(launches * args.steps), "launches_per_step": launches,
            "roofline": roofline, "e2e": e2e}
    if clk:
        line["clocks"] = clk
    if ctx.rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample([sim], [p], 2)
    sim.close()
    return line


# ------------------------------------------------------------------ large
LARGE_SPINUP = 10
LARGE_BUDGET = 100 * 10 ** 9


def run_large(args, ctx):
    """BASELINE config 5: the 512^3 4-level fire plume with a 100 GB block
    budget (which exceeds the full block count of every level, so every level
    is allocated in full), FP16 storage against FP32, and the uniform grid at
    the largest cube that fits the same 100 GB."""
    from dcgrid_gb300 import Simulation, capi, memory, scenes
    out = {}
    sims = [("fp16", capi.PRECISION_MIXED_FP16, capi.MODE_ADAPTIVE), ("fp32", capi.PRECISION_FP32, capi.MODE_ADAPTIVE),
            ("uniform_fp32", capi.PRECISION_FP32, capi.MODE_UNIFORM)]
    clk, launches, roof = None, 0, None
    for name, prec, mode in sims:
        p = scenes.fire(precision=prec, budget_bytes=LARGE_BUDGET)
        if mode == capi.MODE_UNIFORM:
            p.levels = 0
            edge = memory.uniform_edge_for_budget(p, LARGE_BUDGET)
            p.gx = p.gy = p.gz = edge
            p.src_center[0] = p.src_center[2] = edge / 2.0
        s = Simulation(p, mode)
        s.set_stream(ctx.stream.cuda_stream)
        s.add_velocity_noise(0, 0.01)
        s.step(LARGE_SPINUP + max(args.warmup, 3))
        s.sync()
        if name == "fp16":
            clocks = Clocks(ctx.clock_path)
            clocks.start()
        ms, cells = ctx.timed(args.steps, lambda: s.step(1), lambda: s.stats().active_cells, "timed_" + name)
        s.sync()
        if name == "fp16":
            clk = clocks.stop(ctx.local)
            launches = s.launches_per_step()
            peak, peak_kind = peaks()
            jms, jbytes = s.time_kernel(4, 0, 3)
            ach = jbytes / (jms * 1e-3) / 1e9
            roof = {"bound": "hbm", "kernel": f"k_level_solve_batch (one member, level 0, {ITERS} sweeps)",
                    "achieved": ach, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": ach / peak,
                    "traffic": None, "algorithmic_bytes_per_launch": jbytes, "launch_ms": jms}
        ms, cells = ctx.max_sum(ms, cells)
        out[name] = {"value": cells / (ms * 1e-3), "ms_per_step": ms / args.steps, "domain": p.gx,
                     "max_blocks": p.max_blocks if mode == capi.MODE_ADAPTIVE else None,
                     "device_bytes": s.info.device_bytes, "active_cells_per_step": cells / args.steps}
        s.close()
    v = out["fp16"]
    line = {"metric": METRIC, "value": v["value"], "unit": METRIC, "n_gpus": ctx.world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": v["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp16 storage / fp32 compute",
            "data": "synthetic (seeded terrain, jittered heat source, velocity noise)",
            "config": {"workload": "fire plume, effective 512^3, 4 levels, block budget sized to 100 GB "
                                   f"(= the full {v['max_blocks']} blocks), crosswind 2 cells/step, "
                                   f"{ITERS} Jacobi sweeps/level, FP16 scalar storage",
                       "spinup_steps": LARGE_SPINUP, "l2": "inputs larger than L2; flushed between steps",
                       "parallelism": f"replicas x{ctx.world}" if ctx.world > 1 else "single"},
            "comparison": out, "gpu_launches": int(launches * args.steps), "launches_per_step": launches,
            "roofline": roof,
            "cpu_baseline": None,
            "e2e": None}
    if clk:
        line["clocks"] = clk
    return line


# ------------------------------------------------------------------ precision
PRECISION_STEPS = 200
PRECISION_AT = (10, 20, 30, 40, 50, 100, 150, 200)


def run_precision(args, ctx):
    """Per-field error of each storage precision against the FP64 oracle on
    the 3-level cloud scene at effective 256^3 with a 40000-block budget over
    200 steps: FP32, FP16 scalar storage and BF16 scalar storage, each driving
    its own FP64 oracle with the GPU's adaptation decisions (so both sides
    share one topology); relative L2 over the allocated cells after 10, 20, 30,
    40, 50, 100, 150 and 200 steps.
    Not a timing: the line's value is the final FP16 density error."""
    from dcgrid_gb300 import Simulation, capi, scenes
    from oracle import pyoracle
    import numpy as np
    pyoracle.set_threads(os.cpu_count() or 1)
    em = scenes.emission_field(EM_N, 1)
    fields = ["density", "temperature", "vapor", "vel_x", "vel_y", "vel_z", "pressure"]
    out = {}
    t0 = time.perf_counter()
    for name, prec in [("fp32", capi.PRECISION_FP32), ("fp16", capi.PRECISION_MIXED_FP16),
                       ("bf16", capi.PRECISION_MIXED)]:
        p = scenes.cloud256(precision=prec)
        g = Simulation(p)
        g.set_stream(ctx.stream.cuda_stream)
        q = capi.params_from_dict(capi.params_to_dict(p))
        q.precision = capi.PRECISION_FP32
        o = pyoracle.OracleSim(q, precision="double")
        for s in (g, o):
            s.set_emission(em)
            s.add_velocity_noise(0, 0.01)
        rows = []
        for step in range(1, PRECISION_STEPS + 1):
            g.advect_velocity()
            o.advect_velocity()
            g.adapt()
            mv, rf = g.get_last_adapt()
            o.adapt_replay(mv, rf)
            g.project()
            o.project()
            g.advect_scalars()
            o.advect_scalars()
            if step in PRECISION_AT:
                g.sync()
                alloc = np.repeat(o.get_topology()["pos"][:, 3] >= 0, 64)
                row = {"step": step, "active_cells": int(g.stats().active_cells)}
                for f in fields:
                    a = g.get_field(f)[alloc].astype(np.float64)
                    b = o.get_field(f)[alloc]
                    row[f] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
                rows.append(row)
        g.close()
        out[name] = rows
    final = out["fp16"][-1]["density"]
    return {"metric": "relative L2 density error vs FP64 oracle (FP16 storage)", "value": final,
            "unit": "relative L2", "n_gpus": ctx.world, "steps": PRECISION_STEPS, "warmup": 0,
            "higher_is_better": False, "dtype": "fp16/bf16 storage, fp32 compute; fp32",
            "data": "synthetic (seeded terrain, source bubble, emission map, velocity noise)",
            "config": {"workload": "adaptive cloud scene, effective 256^3, 3 levels, 40000 block budget, "
                                   f"{ITERS} Jacobi sweeps/level, {PRECISION_STEPS} steps",
                       "oracle": "FP64, the GPU's adaptation decisions replayed",
                       "cells": "allocated cells of all levels"},
            "errors": out, "wall_s": time.perf_counter() - t0}


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    """--impl reference: the reference's arithmetic on the host cores. The
    reference has no CPU implementation, so its FP64 restatement (the oracle
    port) is timed; each step is one oracle step of every simulation of the
    workload, after a shorter spin-up than the GPU arm's."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import pyoracle
    from dcgrid_gb300 import capi, scenes
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    if args.workload == "batch":
        params = batch_params(capi.PRECISION_FP32)
        ems = [member_emission(i) for i in range(BATCH_N)]
        spin = BATCH_SPINUP
        workload = f"batch of {BATCH_N} independent plumes (same members as the GPU arm), FP64"
    else:
        params = [scenes.cloud256()]
        ems = [scenes.emission_field(EM_N, 1)]
        spin = CLOUD_SPINUP
        workload = "adaptive cloud scene, effective 256^3, 3 levels, 40000 block budget, FP64"
    # the GPU arm's spin-up: the same number of steps before the timed ones
    orcs = []
    for p, e in zip(params, ems):
        o = pyoracle.OracleSim(p, precision="double")
        o.set_emission(e)
        o.add_velocity_noise(0, 0.01)
        o.step(spin + max(args.warmup, 3))
        orcs.append(o)
    cells = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for o in orcs:
            o.step(1)
            cells += o.stats().active_cells
    dt = time.perf_counter() - t0
    warm = max(args.warmup, 3)
    val = cells / dt
    line = {"metric": METRIC, "value": val, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": workload, "spinup_steps": spin, "warmup_steps": warm},
            "cpu_baseline": {"value": val, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} oracle steps of every simulation after {spin} spin-up and "
                                       f"{warm} warm-up steps (the GPU arm's), {threads} OpenMP threads"},
            "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "cloud", "large", "precision"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and FP64 error legs")
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip the reference-kernel GPU comparator")
    ap.add_argument("--profile", action="store_true",
                    help="batch workload: time the headline leg only (for profiler runs)")
    ap.add_argument("--tuning", default=None,
                    help="batch workload: a tuning as JSON (the config.tuning of an earlier line) instead of autotuning")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    ctx = Ctx()
    line = {"batch": run_batch, "cloud": run_cloud, "large": run_large,
            "precision": run_precision}[args.workload](args, ctx)
    if ctx.rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
