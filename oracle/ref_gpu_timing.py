"""Plain GPU comparator (TEST INFRASTRUCTURE): the reference's own CUDA kernels
(oracle/_ref/ref_dcgrid.cubin, built from the reference sources by
oracle/build_ref.sh) run headless on the GPU through oracle/ref_driver.py, and
the GB300-native library on the same input, the reference's default scene
(inlet source, geometric refinement score, derived level count, compat
quirks, 10 Jacobi sweeps per level as hard-wired in
src/dcgrid/fluid_simulation_dcgrid.cu:274-290).

Both paths produce identical fields and topology on this input (pinned by
tests/test_golden.py and tests/test_parity_gpu.py), so their active cell
counts agree and the step rates compare like for like.

Reported per size:
  ref_step_ms        — wall time of one reference step: its kernels plus its
                       host ranking of move/refine candidates (restated in
                       numpy; the reference does it with std::sort on the
                       host) and the device<->host copies around it
  ref_kernels_ms     — the reference's advectVelocity + project +
                       advectDensity stages alone (device-bound kernel
                       sequences, CUDA events on the launch stream)
  ours_step_ms       — dcg_step (one CUDA graph), CUDA events
Usage: python oracle/ref_gpu_timing.py [--steps K]
"""
import argparse
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def run(size, blocks, steps, warmup=3):
    import torch
    from dcgrid_gb300 import Simulation, capi
    from oracle.ref_driver import Driver, RefDCGrid, REF_DIR
    p = capi.default_params(*size, blocks)
    p.jacobi_iters = 10
    drv = Driver(os.path.join(REF_DIR, "ref_dcgrid.cubin"))
    ref = RefDCGrid(drv, p)
    ours = Simulation(p)
    for _ in range(warmup):
        ref.step(1)
        ours.step(1)
    ours.sync()
    torch.cuda.synchronize()
    # reference: whole step (kernels + host ranking) and the kernel-only stages
    t_step, t_kern, cells = 0.0, 0.0, 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(steps):
        t0 = time.perf_counter()
        e0.record()
        ref.advectVelocity()
        e1.record()
        torch.cuda.synchronize()
        k = e0.elapsed_time(e1)
        ref.adaptTopology()
        e0.record()
        ref.project()
        ref.advectDensity()
        e1.record()
        torch.cuda.synchronize()
        k += e0.elapsed_time(e1)
        t_step += (time.perf_counter() - t0) * 1e3
        t_kern += k
    # ours on its own stream, CUDA events on that stream
    st = torch.cuda.Stream()
    ours.set_stream(st.cuda_stream)
    ours_ms = 0.0
    for _ in range(steps):
        e0.record(st)
        ours.step(1)
        e1.record(st)
        torch.cuda.synchronize()
        ours_ms += e0.elapsed_time(e1)
        cells += ours.stats().active_cells
    ours_ms /= steps
    same_topology = bool((ref.snapshot()["level"] != 255).sum() == (ours.get_topology()["pos"][:, 3] >= 0).sum())
    cps = cells / steps
    return {"size": list(size), "max_blocks": blocks, "levels": ref.levels, "sweeps_per_level": 10,
            "steps": steps, "active_cells_per_step": cps,
            "ref_step_ms": t_step / steps, "ref_kernels_ms": t_kern / steps, "ours_step_ms": ours_ms,
            "ref_cell_steps_per_s": cps / (t_step / steps * 1e-3),
            "ref_kernels_cell_steps_per_s": cps / (t_kern / steps * 1e-3),
            "ours_cell_steps_per_s": cps / (ours_ms * 1e-3),
            "speedup_vs_ref_step": (t_step / steps) / ours_ms,
            "speedup_vs_ref_kernels": (t_kern / steps) / ours_ms, "same_block_count": same_topology}


def stage_compare(size, blocks, sweeps, steps=3, warmup=2):
    """Stage-matched GPU times of the reference's kernels and this library on
    the same state (the reference's default scene): advectVelocity,
    adaptTopology (the reference's kernels plus its host ranking),
    project (divergence, cascade, gradient) and advectDensity, each bracketed
    by CUDA events on its side's stream after an L2 flush, averaged over
    `steps` steps; and the whole step (ours: dcg_step's graph). Both sides
    start from the same parameters and make the same decisions, so they hold
    identical states throughout."""
    import torch
    from dcgrid_gb300 import Simulation, capi
    from oracle.ref_driver import Driver, RefDCGrid, REF_DIR
    p = capi.default_params(*size, blocks)
    p.jacobi_iters = sweeps
    drv = Driver(os.path.join(REF_DIR, "ref_dcgrid.cubin"))
    ref = RefDCGrid(drv, p)
    ours = Simulation(p)
    st = torch.cuda.Stream()
    ours.set_stream(st.cuda_stream)
    # the reference launches on the legacy default stream
    streams = (torch.cuda.default_stream(), st)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        ref.step(1)
        ours.step(1)
    ours.sync()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    names = ["advectVelocity", "adaptTopology", "project", "advectDensity"]
    ours_fn = [ours.advect_velocity, ours.adapt, ours.project, ours.advect_scalars]
    ref_fn = [ref.advectVelocity, ref.adaptTopology, ref.project, ref.advectDensity]
    acc = {n: [0.0, 0.0] for n in names}
    for _ in range(steps):
        for k, n in enumerate(names):
            for side, fn in ((0, ref_fn[k]), (1, ours_fn[k])):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                e0.record(streams[side])
                fn()
                e1.record(streams[side])
                torch.cuda.synchronize()
                acc[n][side] += e0.elapsed_time(e1)
    ours.sync()
    stages = {}
    for n in names:
        r, o = acc[n][0] / steps, acc[n][1] / steps
        stages[n] = {"reference_ms": r, "ours_ms": o, "ratio": r / o}
    # whole steps: ours through the captured graph
    step_ms = 0.0
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0.record(st)
        ours.step(1)
        e1.record(st)
        torch.cuda.synchronize()
        step_ms += e0.elapsed_time(e1)
    ref_step = sum(v["reference_ms"] for v in stages.values())
    return {"size": list(size), "max_blocks": blocks, "levels": ref.levels, "sweeps_per_level": sweeps,
            "steps": steps, "stages": stages, "reference_step_ms": ref_step, "ours_graph_step_ms": step_ms / steps,
            "step_ratio": ref_step / (step_ms / steps),
            "same_block_count": bool((ref.snapshot()["level"] != 255).sum() ==
                                     (ours.get_topology()["pos"][:, 3] >= 0).sum())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--stages", action="store_true", help="stage-matched times at 10 and 100 sweeps per level")
    args = ap.parse_args()
    for size, blocks in [((64, 128, 64), 3000), ((256, 256, 256), 40000)]:
        if args.stages:
            for sweeps in (10, 100):
                print(json.dumps(stage_compare(size, blocks, sweeps, args.steps)), flush=True)
        else:
            print(json.dumps(run(size, blocks, args.steps)), flush=True)


if __name__ == "__main__":
    main()
