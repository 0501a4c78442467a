"""Headless renderer, CPU restatement (oracle): the ray march composites the
density volume, shades floor and solids, and draws the debug slice channels
(src/raymarching.cuh). CPU-only sanity checks; GPU parity is in
tests/test_render_gpu.py."""
import numpy as np

from dcgrid_gb300 import capi
from tests import scenarios


def render_params(p, w=48, h=40, channel=capi.RENDER_FLUID, shadows=0, solids=0, precise=1):
    rp = capi.DcgRenderParams()
    rp.width, rp.height = w, h
    rp.eye[0], rp.eye[1], rp.eye[2] = 0.5 * p.gx * p.dx, 0.5 * p.gy * p.dx, -1.2 * p.gz * p.dx
    rp.eye_dir[2] = 1.0
    rp.fov = 0.6
    rp.sun_dir[0], rp.sun_dir[1], rp.sun_dir[2] = 0.4, 0.8, 0.45
    rp.aa_samples = 1
    rp.channel, rp.shadows, rp.solids, rp.precise = channel, shadows, solids, precise
    rp.ambient = 0.3
    for i in range(3):
        rp.smoke_color[i] = 0.9
        rp.scene_color[i] = 0.5
        rp.floor_color[i] = 0.6
    return rp


def plume_state():
    from oracle.pyoracle import OracleSim
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    o = OracleSim(p, precision="float")
    o.add_velocity_noise(1, 0.2)
    o.step(3)
    return p, o


def test_smoke_is_composited_where_the_density_is():
    p, o = plume_state()
    img = o.render(render_params(p))
    assert img.shape == (40, 48, 4) and np.isfinite(img).all()
    alpha = img[..., 3]
    assert alpha.max() > 0.05 and (alpha > 1e-3).sum() < alpha.size
    # the source sits at the bottom centre: smoke in the centre column of the image
    assert alpha[:, 20:28].max() > alpha[:, :6].max()
    rgb = img[..., :3][alpha > 1e-3]
    assert (rgb <= 0.9 + 1e-5).all() and (rgb >= 0.3 * 0.9 - 1e-5).all()  # ambient .. full light


def test_debug_channels():
    p, o = plume_state()
    res = o.render(render_params(p, channel=capi.RENDER_RESOLUTION))
    vals = np.unique(np.round(res[..., 0][res[..., 3] > 0], 6))
    assert set(vals) <= {0.0, 1.0} and len(vals) == 2
    dens = o.render(render_params(p, channel=capi.RENDER_DENSITY))
    assert dens[..., 0].max() > 0 and np.allclose(dens[..., 1:3], 0)
    flu = o.render(render_params(p, channel=capi.RENDER_FLUIDITY))
    seen = flu[..., 3] > 0
    assert np.allclose(flu[..., 0][seen], 1.0)  # no solids: fluidity 1 everywhere


def test_floor_and_shadows():
    p, o = plume_state()
    lit = o.render(render_params(p, solids=1, shadows=0))
    shadowed = o.render(render_params(p, solids=1, shadows=1))
    assert (lit[..., 3] > 0.99).any()  # the floor is opaque
    assert shadowed[..., :3].sum() <= lit[..., :3].sum() + 1e-6
