"""Host calls a step depends on, on the GPU.

* dcg_set_params (the reference's copySimParamsToDevice, per handle): a
  physics change takes effect in captured step graphs (graph replay equals
  stage calls after the change, and differs from the unchanged run);
  geometry, budget and odd sweep counts are refused.
* dcg_set_stream: steps on a caller's stream give the same results.
* dcg_time_kernel, dcg_launches_per_step, dcg_batch_get_tuning: report
  positive times, algorithmic bytes and launch counts.
"""
import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios
from tests.test_parity_gpu import compare

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib")]


def plume():
    return scenarios.plume(32, 64, 32, None, 2, 10)


def test_set_params_takes_effect_in_captured_steps():
    from dcgrid_gb300 import Simulation
    p = plume()
    a, b, c = Simulation(p), Simulation(p), Simulation(p)
    b.set_graphs(False)
    for s in (a, b, c):
        s.add_velocity_noise(2, 0.3)
        s.step(2)
    q = plume()
    q.dt, q.buoy_beta = 0.05, 0.6
    for s in (a, b):
        s.set_params(q)
    for s in (a, b, c):
        s.step(2)
        s.sync()
    compare(a, b, q, "graph replay after set_params vs stage calls")
    assert not np.array_equal(a.get_field("vel_y"), c.get_field("vel_y"))


def test_set_params_refuses_fixed_fields():
    from dcgrid_gb300 import DcgError, Simulation
    s = Simulation(plume())
    for change in [("max_blocks", plume().max_blocks + 8), ("gx", 64), ("n_scalars", 1), ("jacobi_iters", 7),
                   ("precision", capi.PRECISION_MIXED_FP16)]:
        q = plume()
        setattr(q, *change)
        with pytest.raises(DcgError) as e:
            s.set_params(q)
        assert e.value.code == capi.DCG_E_INVALID, change


def test_caller_stream_gives_the_same_results():
    import torch
    from dcgrid_gb300 import Simulation
    p = plume()
    a, b = Simulation(p), Simulation(p)
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    for s in (a, b):
        s.add_velocity_noise(3, 0.2)
        s.step(3)
        s.sync()
    compare(a, b, p, "caller's stream")


def test_kernel_timing_and_launch_counts():
    from dcgrid_gb300 import Batch, Simulation
    s = Simulation(plume())
    s.step(1)
    assert s.launches_per_step() > 0
    for which in (0, 1, 2, 3, 4):  # Jacobi sweep, advections, divergence, level solve
        ms, nbytes = s.time_kernel(which, 0, 3)
        assert ms > 0 and nbytes > 0, which
    b = Batch(scenarios.plume_batch(2, 1, sizes=(16, 32), iters=10))
    t = b.get_tuning()
    assert all(x in (1, 2, 4, 8) for x in t.tile) and t.solve_cache in (0, 3, 4, 8, 16, 18, 19, 32, 34, 35, 64, 66, 83)
