"""Parity at the sizes the benchmark configurations are stated at.

* Smoke plume, effective 64x128x64, 2 levels of 4^3-cell blocks, sphere source
  r=6 at (32, 6, 32) with density 1 and temperature +10, buoyancy alpha=0.1
  beta=0.3, dt=0.1, 100 Jacobi sweeps per level, closed walls, seed-0 velocity
  noise of amplitude 0.01, 50 steps: the GPU step equals the oracle's float
  mirror bit for bit, compared every 10 steps (block table and every field),
  and the FP32 path stays within 1e-4 relative L2 of the FP64 oracle per field
  (the FP64 oracle replays the GPU's adaptation decisions).
* Cloud, effective 256^3, 3 levels, 40000-block budget, terrain, wind inflow,
  three scalars, field-driven refinement, 100 sweeps: from creation the GPU
  and the oracle's float mirror stay bit-identical after every one of 12
  steps; after a GPU spin-up the float mirror takes over the GPU state, and
  for the next steps both step independently and stay bit-identical.
* Largest plume of the benchmark batch (256^3, FP16 storage): density error
  against the FP64 oracle at the benchmark's horizon (spin-up + timed steps).
"""
import numpy as np
import pytest

from dcgrid_gb300 import capi, scenes
from tests.test_parity_gpu import compare, field_names

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib", "oracle_lib")]


def _oracle(p, prec):
    from oracle.pyoracle import OracleSim
    return OracleSim(p, precision=prec)


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def plume_64x128x64():
    p = scenes.plume(64, 128, 64, None, 2, 100)
    assert (p.src_center[0], p.src_center[1], p.src_center[2], p.src_radius) == (32.0, 6.0, 32.0, 6.0)
    assert (p.buoy_alpha, p.src_temperature, p.src_density, p.jacobi_iters) == (pytest.approx(0.1), 10.0, 1.0, 100)
    return p


def test_plume_64x128x64_50_steps_bitexact_every_10_steps():
    from dcgrid_gb300 import Simulation
    p = plume_64x128x64()
    g, o = Simulation(p), _oracle(p, "float")
    for s in (g, o):
        s.add_velocity_noise(0, 0.01)
    for k in range(5):
        g.step(10)
        o.step(10)
        g.sync()
        compare(g, o, p, f"after {10 * (k + 1)} steps")
    st = g.stats()
    assert st.device_error == 0 and st.active_cells > 64 * 128 * 64 // 8


def test_plume_64x128x64_50_steps_fp32_vs_fp64():
    from dcgrid_gb300 import Simulation
    p = plume_64x128x64()
    g, d = Simulation(p), _oracle(p, "double")
    for s in (g, d):
        s.add_velocity_noise(0, 0.01)
    errs = {}
    for step in range(50):
        g.advect_velocity()
        d.advect_velocity()
        g.adapt()
        mv, rf = g.get_last_adapt()
        d.adapt_replay(mv, rf)
        g.project()
        d.project()
        g.advect_scalars()
        d.advect_scalars()
    g.sync()
    alloc = np.repeat(d.get_topology()["pos"][:, 3] >= 0, 64)
    for f in ["density", "temperature", "vel_x", "vel_y", "vel_z", "pressure"]:
        errs[f] = _rel_l2(g.get_field(f)[alloc].astype(np.float64), d.get_field(f)[alloc])
    print("FP32 vs FP64 relative L2 after 50 steps:", errs)
    assert all(e <= 1e-4 for e in errs.values()), errs


def test_cloud256_40k_blocks_spun_up_window_bitexact():
    from dcgrid_gb300 import Simulation
    p = scenes.cloud256()
    g = Simulation(p)
    em = scenes.emission_field(16, 1)
    g.set_emission(em)
    g.add_velocity_noise(0, 0.01)
    g.step(40)
    g.sync()
    # the oracle takes over the GPU's spun-up state (block table and fields)
    o = _oracle(p, "float")
    o.set_emission(em)
    o.set_topology(g.get_topology())
    for f in field_names(p):
        o.set_field(f, g.get_field(f))
    compare(g, o, p, "after the state copy")
    moved = 0
    for k in range(4):
        g.step(1)
        o.step(1)
        g.sync()
        compare(g, o, p, f"spun-up step {k + 1}")
        moved += g.stats().moved_blocks + g.stats().refined_subblocks
    assert g.stats().active_cells > 500_000
    assert moved > 0  # the window includes topology changes


@pytest.mark.parametrize("compat", [0, 1])
def test_cloud256_40k_blocks_from_creation_bitexact_every_step(compat):
    """The same cloud from creation: GPU and float mirror step independently
    for 12 steps and stay bit-identical after every step. The early steps
    move blocks next to coarser levels while refining heavily, so the
    rescoring after the moves must see a moved block's neighbours as the
    not yet refreshed neighbour indices give them (from its old place). With
    ref_compat the neighbour refresh after step 9 keeps the reference's
    entries that point one level too coarse (a block moved in and refined in
    the same adaptation); without it every entry is the finest block's."""
    from dcgrid_gb300 import Simulation
    p = scenes.cloud256()
    p.ref_compat = compat
    g, o = Simulation(p), _oracle(p, "float")
    em = scenes.emission_field(16, 1)
    for s in (g, o):
        s.set_emission(em)
        s.add_velocity_noise(0, 0.01)
    moved = 0
    for k in range(12):
        g.step(1)
        o.step(1)
        g.sync()
        compare(g, o, p, f"step {k + 1}")
        moved += g.stats().moved_blocks
    assert moved > 0


def test_largest_batch_member_fp16_density_error_at_bench_horizon():
    """The 256^3 member of the benchmark batch with FP16 scalar storage, over
    the benchmark's 30 spin-up + 3 warm-up + 10 timed steps, against the FP64
    oracle driven with the GPU's adaptation decisions: density within 1e-3."""
    from dcgrid_gb300 import Simulation
    params = scenes.plume_batch(16, 0, sizes=(64, 96, 128, 192, 256), iters=100,
                                precision=capi.PRECISION_MIXED_FP16, em_n=16)
    i = max(range(16), key=lambda k: params[k].max_blocks)
    p = params[i]
    assert p.gx == 256
    g = Simulation(p)
    q = capi.params_from_dict(capi.params_to_dict(p))
    q.precision = capi.PRECISION_FP32
    d = _oracle(q, "double")
    em = scenes.emission_field(16, 100 + i)
    for s in (g, d):
        s.set_emission(em)
        s.add_velocity_noise(0, 0.01)
    for step in range(43):
        g.advect_velocity()
        d.advect_velocity()
        g.adapt()
        mv, rf = g.get_last_adapt()
        d.adapt_replay(mv, rf)
        g.project()
        d.project()
        g.advect_scalars()
        d.advect_scalars()
    g.sync()
    alloc = np.repeat(d.get_topology()["pos"][:, 3] >= 0, 64)
    err = {f: _rel_l2(g.get_field(f)[alloc].astype(np.float64), d.get_field(f)[alloc])
           for f in ["density", "temperature", "vel_y", "pressure"]}
    print(f"member {i} ({p.gx}^3, {p.levels} levels), 43 steps, FP16 storage vs FP64:", err)
    assert err["density"] <= 1e-3, err
