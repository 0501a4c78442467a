"""Headless renderer on the GPU against its CPU restatement (oracle float
mirror) on identical states. The fields are bit-identical (stage parity), the
march takes the same steps; exponentials are computed by different libraries,
so images are compared with a tolerance."""
import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios
from tests.test_parity_gpu import gpu, orc
from tests.test_render_oracle import render_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib", "oracle_lib")]


def pair(p, mode=capi.MODE_ADAPTIVE, steps=3):
    g, o = gpu(p, mode), orc(p, "float", mode)
    for s in (g, o):
        s.add_velocity_noise(1, 0.2)
        s.step(steps)
    g.sync()
    return g, o


def close(a, b, where):
    d = np.abs(a.astype(np.float64) - b)
    assert np.median(d) < 1e-6, where
    assert (d > 1e-4).mean() < 1e-3, (where, float(d.max()), float((d > 1e-4).mean()))


CASES = {
    "fluid": dict(channel=capi.RENDER_FLUID),
    "fluid_shadows_solids": dict(channel=capi.RENDER_FLUID, shadows=1, solids=1),
    "coarse": dict(channel=capi.RENDER_FLUID, precise=0),
    "density": dict(channel=capi.RENDER_DENSITY),
    "velocity": dict(channel=capi.RENDER_VELOCITY),
    "fluidity": dict(channel=capi.RENDER_FLUIDITY),
    "resolution": dict(channel=capi.RENDER_RESOLUTION),
}


@pytest.mark.parametrize("case", list(CASES))
def test_adaptive_render_matches_cpu(case):
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    g, o = pair(p)
    rp = render_params(p, **CASES[case])
    close(g.render(rp), o.render(rp), case)


@pytest.mark.parametrize("compat", [1, 0])
def test_sphere_scene_and_coarse_sampling_quirk(compat):
    p = scenarios.sphere_obstacle(32, 64, 32, 600)
    p.ref_compat = compat
    g, o = pair(p)
    for kw in [dict(channel=capi.RENDER_FLUID, solids=1, shadows=1), dict(channel=capi.RENDER_DENSITY, precise=0)]:
        rp = render_params(p, **kw)
        close(g.render(rp), o.render(rp), (compat, kw))


def test_uniform_render_matches_cpu():
    p = scenarios.plume(32, 64, 32, None, 0, 10)
    p.levels = 0
    g, o = pair(p, capi.MODE_UNIFORM)
    for kw in [dict(channel=capi.RENDER_FLUID, shadows=1, solids=1), dict(channel=capi.RENDER_VELOCITY),
               dict(channel=capi.RENDER_FLUID, precise=0)]:
        rp = render_params(p, **kw)
        close(g.render(rp), o.render(rp), kw)


def test_render_into_device_memory():
    import torch
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    g, _ = pair(p)
    rp = render_params(p, shadows=1)
    host = g.render(rp)
    dev = g.render(rp, torch.empty((rp.height, rp.width, 4), dtype=torch.float32, device="cuda"))
    assert np.array_equal(dev.cpu().numpy(), host)
