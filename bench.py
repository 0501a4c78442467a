"""Benchmark of the adaptive-grid simulation step on GB300.

Metric: active (leaf) cell-steps per second of the 3-level adaptive cloud scene
(effective 256^3 domain, 40k-block budget, terrain SDF from 5-octave value
noise, wind inflow of 1 cell/step, temperature/vapor/density, refinement by
|curl v| > 0.5 or |grad rho| > 0.05), 100 Jacobi sweeps per level.
Synthetic inputs: seeded terrain, a seeded warm moist source bubble, seeded
velocity noise; the scene is spun up 60 untimed steps before warm-up so the
refined topology is developed.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun with N > 1 every rank runs an independent replica of the scene
(one simulation does not shard); value sums the ranks' cell-steps over the
slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

G = 256
BLOCKS = 40000
LEVELS = 3
ITERS = 100
SPINUP = 60
EM_N = 16


def workload_params(precision="fp32"):
    from dcgrid_gb300 import capi
    p = capi.default_params(G, G, G, BLOCKS)
    p.levels = LEVELS
    p.dx = 1.0
    p.dt = 1.0
    p.inlet_enabled = 0
    p.jacobi_iters = ITERS
    p.n_scalars = 3
    p.buoy_alpha = 0.1
    p.buoy_beta = 0.3
    p.t_ambient = 0.0
    p.solids = capi.SOLIDS_TERRAIN
    p.terrain_amplitude = 40.0
    p.terrain_base_height = 8.0
    p.terrain_frequency = 1.0 / 64.0
    p.terrain_persistence = 0.5
    p.terrain_octaves = 5
    p.terrain_seed = 7
    p.wind_enabled = 1
    p.wind[0] = 1.0
    p.refine_criterion = capi.REFINE_FIELDS
    p.refine_threshold = 1.0
    p.vort_threshold = 0.5
    p.grad_threshold = 0.05
    p.ref_compat = 0
    p.src_enabled = 1
    p.src_center[0] = 0.3 * G
    p.src_center[1] = 0.25 * G
    p.src_center[2] = 0.5 * G
    p.src_radius = 16.0
    p.src_density = 1.0
    p.src_temperature = 5.0
    p.src_vapor = 0.5
    p.precision = capi.PRECISION_FP32 if precision == "fp32" else capi.PRECISION_MIXED
    p.emission_n = EM_N
    p.emission_band = 16.0
    return p


def emission_field(seed=1):
    """Seeded ground emission (density per time unit), EM_N^3 values in [0, 0.05)."""
    import numpy as np
    return (0.05 * np.random.default_rng(seed).random(EM_N ** 3)).astype(np.float32)


CONFIG = {"workload": f"adaptive cloud scene, effective {G}^3, {LEVELS} levels, {BLOCKS} block budget, "
                      f"{ITERS} Jacobi sweeps/level",
          "domain": [G, G, G], "levels": LEVELS, "max_blocks": BLOCKS, "jacobi_iters": ITERS,
          "block_edge": 4, "spinup_steps": SPINUP, "n_scalars": 3,
          "emission": f"{16}^3 field over the bottom 16 cell layers",
          "l2": "flushed between timed steps (256 MiB write)"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch():
    """dram bytes of one Jacobi launch from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "jacobi_traffic.json")) as f:
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


def cpu_baseline(gpu_sim=None, steps=1):
    """The FP64 oracle on the host cores: `steps` steps of the same workload,
    started from the GPU's spun-up state when given (topology and fields)."""
    from oracle import pyoracle
    from dcgrid_gb300 import capi
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    p = workload_params()
    o = pyoracle.OracleSim(p, precision="double")
    o.set_emission(emission_field())
    if gpu_sim is not None:
        topo = gpu_sim.get_topology()
        o.set_topology(topo)
        names = ["density", "temperature", "vapor", "vel_x", "vel_y", "vel_z", "fluidity"]
        for f in names:
            o.set_field(f, gpu_sim.get_field(f).astype("float64"))
    else:
        o.add_velocity_noise(0, 0.01)
        o.step(SPINUP)
    cells = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step(1)
        cells += o.stats().active_cells
    dt = time.perf_counter() - t0
    return {"value": cells / dt, "unit": "active cell-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} step(s) of the same workload from the spun-up state, FP64 oracle, "
                      f"{threads} OpenMP threads"}, o


def run_reference(args):
    """--impl reference: the reference's own arithmetic on the host cores (the
    reference has no CPU implementation and its GPU kernels are not the CPU arm;
    the oracle port is timed), each step one oracle step of the same workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    p = workload_params()
    o = pyoracle.OracleSim(p, precision="double")
    o.set_emission(emission_field())
    o.add_velocity_noise(0, 0.01)
    o.step(SPINUP)
    for _ in range(args.warmup):
        o.step(1)
    cells = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(1)
        cells += o.stats().active_cells
    dt = time.perf_counter() - t0
    val = cells / dt
    line = {"metric": "active cell-steps/s", "value": val, "unit": "active cell-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference", "config": CONFIG,
            "cpu_baseline": {"value": val, "unit": "active cell-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} oracle steps after {SPINUP} spin-up and {args.warmup} "
                                       f"warm-up steps, {threads} OpenMP threads"},
            "e2e": {"value": val, "unit": "active cell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from dcgrid_gb300 import Simulation, build
    build.build()
    stream = torch.cuda.Stream()
    p = workload_params()
    sim = Simulation(p)
    sim.set_stream(stream.cuda_stream)
    em = emission_field()
    sim.set_emission(em)
    sim.add_velocity_noise(0, 0.01)
    sim.step(SPINUP)
    for _ in range(max(args.warmup, 3)):
        sim.step(1)
    sim.sync()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # ---- device-resident timed region
    clocks = Clocks(os.path.join(ROOT, "gpurun_out", f"clocks_r{rank}.csv")
                    if os.path.isdir(os.path.join(ROOT, "gpurun_out")) else f"/tmp/dcg_clocks_r{rank}.csv")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    cells = 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        ev[k][0].record(stream)
        sim.step(1)
        ev[k][1].record(stream)
        cells += sim.stats().active_cells
    torch.cuda.synchronize()
    clk = clocks.stop(local)
    ms = sum(a.elapsed_time(b) for a, b in ev)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        c = torch.tensor([float(cells)], device="cuda")
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        cells = float(c.item())
    value = cells / (ms * 1e-3)
    launches = sim.launches_per_step()

    # ---- end to end through the public API: per step the host uploads the
    # step's emission field (pinned host -> device, dcg_set_emission) and reads
    # back the dense density volume the step produced (device -> pinned host).
    n_dense = G * G * G
    host_out = torch.empty(n_dense, dtype=torch.float32).pin_memory()
    host_em = torch.from_numpy(em).pin_memory()
    import ctypes as C
    from dcgrid_gb300 import capi
    e2e_ms = 0.0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e2e_cells = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        sim.set_emission(host_em)
        sim.step(1)
        rc = sim.L.dcg_get_dense(sim.h, capi.FIELD_DENSITY, C.c_void_p(host_out.data_ptr()), capi.HOST)
        if rc:
            raise RuntimeError("dcg_get_dense failed")
        e2e_cells += sim.stats().active_cells
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3
    if dist:
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
        c = torch.tensor([float(e2e_cells)], device="cuda")
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        e2e_cells = float(c.item())
    e2e = {"value": e2e_cells / (e2e_ms * 1e-3), "unit": "active cell-steps/s",
           "h2d_bytes_per_step": 4 * EM_N ** 3, "d2h_bytes_per_step": 4 * n_dense,
           "note": "per step: dcg_set_emission from pinned host memory, dcg_step, dcg_get_dense into pinned "
                   "host memory, dcg_get_stats; host clock"}

    # ---- roofline of the dominant kernel: the cooperative solve of the finest
    # level (one launch = all ITERS sweeps; 12 B per allocated cell per sweep)
    peak, peak_kind = peaks()
    jac_ms, jac_bytes = sim.time_kernel(4, 0, 5)
    achieved = jac_bytes / (jac_ms * 1e-3) / 1e9
    tr = traffic_per_launch()
    roofline = {"bound": "hbm", "kernel": f"k_level_solve (level 0, {ITERS} sweeps per launch)",
                "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": achieved / peak, "traffic": (tr or {}).get("bytes_per_launch_scaled"),
                "algorithmic_bytes_per_launch": jac_bytes, "launch_ms": jac_ms,
                "note": "working set (p, p~, div of the level) is L2-resident across sweeps; frac > 1 "
                        "would mean L2 reuse beyond the HBM roofline"}

    st = sim.stats()
    line = {"metric": "active cell-steps/s", "value": value, "unit": "active cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded terrain, source bubble, velocity noise)",
            "config": dict(CONFIG, parallelism=f"replicas x{world}" if world > 1 else "single",
                           active_cells_last_step=int(st.active_cells)),
            "gpu_launches": int(launches * args.steps), "launches_per_step": launches,
            "roofline": roofline, "e2e": e2e}
    if clk:
        line["clocks"] = clk
    if rank == 0 and not args.no_cpu:
        cb, _ = cpu_baseline(sim, steps=2)
        line["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    sim.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
