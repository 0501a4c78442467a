"""The reference-named host classes on the GPU.

* FluidSimulationDCGrid(size, maxNumBlocks) with the reference's defaults,
  init(), then the reference's per-frame order advectVelocity, adaptTopology,
  project, advectDensity (src/simulation.cpp:104-112): bit-exact against the
  oracle's float mirror.
* reset() after stepping returns to the state creation gives: the same steps
  from there give bit-identical fields and block tables.
* render(dest, resolution, eyePos, eyeDir, fov, sunDir) is dcg_render with
  those camera inputs and the reference's default switches.
"""
import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios
from tests.test_parity_gpu import compare, orc

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib", "oracle_lib")]


def update(sim):
    sim.advectVelocity()
    sim.adaptTopology()
    sim.project()
    sim.advectDensity()


def test_reference_frame_order_matches_oracle():
    from dcgrid_gb300 import FluidSimulationDCGrid
    g = FluidSimulationDCGrid((32, 64, 32), 600)
    g.init()
    p = scenarios.ref_default(32, 64, 32, 600)
    assert capi.params_to_dict(g.params) == pytest.approx(capi.params_to_dict(p))
    o = orc(p)
    for k in range(3):
        update(g)
        o.step(1)
        g.sync()
        compare(g, o, p, f"frame {k}")


def test_reset_returns_to_the_created_state():
    from dcgrid_gb300 import Simulation
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    a, b = Simulation(p), Simulation(p)
    a.add_velocity_noise(3, 0.5)
    a.step(4)
    a.reset()
    for s in (a, b):
        s.add_velocity_noise(5, 0.2)
        s.step(3)
        s.sync()
    compare(a, b, p, "reset vs created")
    assert a.stats().steps == b.stats().steps == 3


def test_reference_render_signature_equals_dcg_render():
    from dcgrid_gb300 import FluidSimulationDCGrid
    from dcgrid_gb300.sim import default_render_params
    g = FluidSimulationDCGrid((32, 64, 32), 600)
    update(g)
    p = g.params
    eye = (0.5 * p.gx * p.dx, 0.5 * p.gy * p.dx, -1.2 * p.gz * p.dx)
    view, sun = (0.0, 1.0, 0.0), (0.3, 0.9, 0.3)
    img = g.render(None, (48, 40), eye, view, 1.1, sun, channel=capi.RENDER_DENSITY)
    rp = default_render_params(48, 40)
    for i in range(3):
        rp.eye[i], rp.eye_dir[i], rp.sun_dir[i] = eye[i], view[i], sun[i]
    rp.fov, rp.channel = 1.1, capi.RENDER_DENSITY
    ref = g.render(rp)
    assert img.shape == (40, 48, 4) and np.isfinite(img).all()
    assert np.array_equal(img, ref)
