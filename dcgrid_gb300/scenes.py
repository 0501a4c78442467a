"""Scene builders: the reference's default scene and the benchmark scenes
(smoke plume, terrain cloud, batches of uneven plumes) as dcg_params, plus
seeded emission maps. Terrain comes from seeded value noise evaluated on the
device (src/noise.cpp:20-107 inspired; the reference's Noise has no seed), or
from a heightmap (dcg_set_heightmap) such as the seeded one built here."""
import random

import numpy as np

from . import capi


def ref_default(gx=32, gy=64, gz=32, blocks=600, solids=capi.SOLIDS_NONE):
    """The reference's defaults (src/data/sim_params.cpp:4-34): bottom inlet,
    geometric refinement score, derived level count, compat quirks on."""
    p = capi.default_params(gx, gy, gz, blocks)
    p.solids = solids
    return p


def plume(gx=32, gy=64, gz=32, blocks=None, levels=2, iters=20):
    """Smoke plume: sphere source (density 1, temperature 10) near the bottom
    centre, buoyancy alpha=0.1 beta=0.3, dt=0.1, closed walls, dx=1."""
    full1 = (gx // 8) * (gy // 8) * (gz // 8)
    full0 = (gx // 4) * (gy // 4) * (gz // 4)
    if blocks is None:
        blocks = full1 + full0 // 2
    p = capi.default_params(gx, gy, gz, blocks)
    p.levels = levels
    p.dx = 1.0
    p.dt = 0.1
    p.inlet_enabled = 0
    p.jacobi_iters = iters
    p.n_scalars = 3
    p.buoy_alpha = 0.1
    p.buoy_beta = 0.3
    p.t_ambient = 0.0
    p.src_enabled = 1
    p.src_center[0] = gx / 2.0
    p.src_center[1] = 6.0
    p.src_center[2] = gz / 2.0
    p.src_radius = 6.0
    p.src_density = 1.0
    p.src_temperature = 10.0
    p.src_vapor = 0.0
    return p


def cloud(g=64, blocks=1500, levels=3, iters=20, compat=0):
    """Cloud scene: terrain SDF from 5-octave value noise, wind inflow at x=0,
    temperature/vapor/density, field-driven refinement (|curl v|, |grad rho|)."""
    p = capi.default_params(g, g, g, blocks)
    p.levels = levels
    p.dx = 1.0
    p.dt = 1.0
    p.inlet_enabled = 0
    p.jacobi_iters = iters
    p.n_scalars = 3
    p.buoy_alpha = 0.1
    p.buoy_beta = 0.3
    p.solids = capi.SOLIDS_TERRAIN
    p.terrain_amplitude = 40.0 * g / 256.0
    p.terrain_base_height = 2.0
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
    p.ref_compat = compat
    p.src_enabled = 1
    p.src_center[0] = g * 0.3
    p.src_center[1] = g * 0.45
    p.src_center[2] = g * 0.5
    p.src_radius = g / 16.0
    p.src_density = 1.0
    p.src_temperature = 5.0
    p.src_vapor = 0.5
    return p


def sphere_obstacle(gx=32, gy=64, gz=32, blocks=600):
    """The reference's SPGridCmp switches: sphere solid on (scenes.h:23-31)."""
    p = capi.default_params(gx, gy, gz, blocks)
    p.solids = capi.SOLIDS_SPHERE
    p.sphere_radius_world = 2000.0
    return p


def plume_batch(n=16, seed=0, sizes=(64, 96, 128, 192, 256), iters=100, precision=capi.PRECISION_FP32,
                levels=(2, 3), em_n=0):
    """Independent plumes with uneven domains: edge drawn from `sizes`, 2 or 3
    levels, a sphere source in the bottom quarter of radius U[4,10] (capped to
    the domain) and temperature U[5,15], field-driven refinement. Budget: the
    coarsest level in full plus a quarter of the finest level's blocks. With
    em_n > 0 each member also takes an em_n^3 emission map over its bottom 16
    cell layers."""
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        d = rng.choice(sizes)
        lv = rng.choice(levels)
        full = [(d >> (l + 2)) ** 3 for l in range(lv)]
        p = plume(d, d, d, full[-1] + full[0] // 4, lv, iters)
        r = min(rng.uniform(4.0, 10.0), d / 8.0)
        p.src_radius = r
        p.src_center[0] = rng.uniform(r, d - r)
        p.src_center[1] = rng.uniform(r, max(r, d / 4.0))
        p.src_center[2] = rng.uniform(r, d - r)
        p.src_temperature = rng.uniform(5.0, 15.0)
        p.refine_criterion = capi.REFINE_FIELDS
        p.refine_threshold = 1.0
        p.vort_threshold = 0.5
        p.grad_threshold = 0.05
        p.ref_compat = 0
        p.precision = precision
        if em_n > 0:
            p.emission_n = em_n
            p.emission_band = 16.0
        out.append(p)
    return out


def cloud256(precision=capi.PRECISION_FP32, blocks=40000, levels=3, iters=100, em_n=16):
    """The 3-level cloud scene at effective 256^3 with a 40k-block budget:
    terrain amplitude 40 cells, wind inflow of 1 cell/step, temperature/vapor/
    density, refinement by |curl v| > 0.5 or |grad rho| > 0.05, and an
    em_n^3 ground emission map over the bottom 16 cell layers."""
    g = 256
    p = cloud(g, blocks, levels, iters, 0)
    p.terrain_amplitude = 40.0
    p.terrain_base_height = 8.0
    p.t_ambient = 0.0
    p.src_center[0] = 0.3 * g
    p.src_center[1] = 0.25 * g
    p.src_center[2] = 0.5 * g
    p.src_radius = 16.0
    p.src_temperature = 5.0
    p.src_vapor = 0.5
    p.precision = precision
    p.emission_n = em_n
    p.emission_band = 16.0
    return p


def heightmap(nx=48, nz=40, seed=0, waves=3):
    """Seeded (nz, nx) float32 heightmap in [0, 1] for dcg_set_heightmap: a sum
    of `waves` plane waves with random wave vectors (1 to 4 periods across the
    map) and phases, rescaled to [0, 1]."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) / nx
    z = (np.arange(nz) + 0.5) / nz
    X, Z = np.meshgrid(x, z)
    h = np.zeros_like(X)
    for _ in range(waves):
        kx, kz = rng.uniform(1.0, 4.0, 2)
        h += np.sin(2.0 * np.pi * (kx * X + kz * Z) + rng.uniform(0.0, 2.0 * np.pi))
    return ((h - h.min()) / (h.max() - h.min())).astype(np.float32)


def emission_field(n=16, seed=1, scale=0.05):
    """Seeded emission map (density per time unit), n^3 values in [0, scale)."""
    return (scale * np.random.default_rng(seed).random(n ** 3)).astype(np.float32)


def differentiable(g=128, levels=2, iters=20, em_n=16, noise=0.5):
    """Differentiable scene: passive density transport in a seeded noise flow
    (no buoyancy, no source, closed walls), the density injected by an
    em_n^3 emission map over the bottom 16 cell layers, and the reference's
    position-based refinement score, so the block topology does not depend on
    the density. Budget: the coarsest level in full plus a quarter of the
    finest level. `noise` is the amplitude of the seeded initial velocity."""
    full = [(g >> (l + 2)) ** 3 for l in range(levels)]
    p = capi.default_params(g, g, g, full[-1] + full[0] // 4)
    p.levels = levels
    p.dx = 1.0
    p.dt = 1.0
    p.inlet_enabled = 0
    p.jacobi_iters = iters
    p.n_scalars = 1
    p.refine_criterion = capi.REFINE_GEOMETRIC
    p.ref_compat = 0
    p.emission_n = em_n
    p.emission_band = 16.0
    return p


def fire(g=512, levels=4, precision=capi.PRECISION_FP32, budget_bytes=100 * 10 ** 9, iters=100):
    """Large fire plume: effective g^3, `levels` levels, block budget sized to
    `budget_bytes` of device memory (dcg_blocks_for_budget; capped at the full
    block count, which 100 GB exceeds at 512^3), terrain from seeded value
    noise (amplitude 40 cells), a ground heat source 64 cells wide at the
    domain centre (temperature 30 with seeded per-cell jitter of +-3, density
    1), buoyancy, crosswind of 2 cells/step, field-driven refinement."""
    from . import memory
    p = cloud(g, 1, levels, iters, 0)
    p.terrain_amplitude = 40.0
    p.terrain_base_height = 4.0
    p.terrain_seed = 13
    p.wind[0] = 2.0
    p.src_center[0] = g / 2.0
    p.src_center[1] = 4.0
    p.src_center[2] = g / 2.0
    p.src_radius = 32.0
    p.src_density = 1.0
    p.src_temperature = 30.0
    p.src_vapor = 0.0
    p.src_jitter = 3.0
    p.src_jitter_seed = 11
    p.precision = precision
    p.max_blocks = memory.blocks_for_budget(p, budget_bytes)
    return p
