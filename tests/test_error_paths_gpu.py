"""Error paths of the device side, without faulting or hanging the GPU.

* Non-finite values: a NaN in a leaf cell's pressure, density or fluidity is
  flagged by the statistics pass (DCG_DEVERR_NAN); dcg_get_stats and dcg_sync
  return DCG_E_NAN, batches likewise. The reference has no such check: it
  exits only on CUDA errors (include/cuda/helper_cuda.h:761-790).
* Bounded waits: dcg_check_barrier_timeout makes the grid barrier of the level
  solves wait on a word that nothing advances; the wait gives up after a short
  poll limit, sets DCG_DEVERR_TIMEOUT, dcg_sync returns DCG_E_DEVICE, and the
  handle keeps working after dcg_reset.
"""
import ctypes as C

import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib")]


def _stats_rc(sim):
    st = capi.DcgStats()
    rc = sim.L.dcg_get_stats(sim.h, C.byref(st))
    return rc, st


def _leaf_cell(sim):
    """index of an allocated leaf cell (block-major layout)"""
    topo = sim.get_topology()
    pos, child = topo["pos"], topo["child"]
    for b in range(len(pos)):
        if pos[b, 3] >= 0 and child[b, 0] == 0xFFFFFFFF:
            return b * 64
    raise AssertionError("no leaf block")


def test_nan_in_pressure_is_reported():
    from dcgrid_gb300 import Simulation
    sim = Simulation(scenarios.plume(32, 64, 32, None, 2, 10))
    sim.step(2)
    rc, st = _stats_rc(sim)
    assert rc == capi.DCG_OK and st.device_error == 0
    assert sim.L.dcg_sync(sim.h) == capi.DCG_OK
    p = sim.get_field("pressure")
    p[_leaf_cell(sim)] = np.nan
    sim.set_field("pressure", p)
    rc, st = _stats_rc(sim)
    assert rc == capi.DCG_E_NAN
    assert st.device_error == capi.DEVERR_NAN and st.active_cells > 0  # filled all the same
    assert "non-finite" in sim.L.dcg_last_error_string(sim.h).decode()
    assert sim.L.dcg_sync(sim.h) == capi.DCG_E_NAN
    sim.reset()
    rc, st = _stats_rc(sim)
    assert rc == capi.DCG_OK and st.device_error == 0


def test_nan_produced_by_a_step_is_reported():
    # a NaN density in a passive-scalar scene spreads through the advection
    # (positions and velocity stay finite) and shows in the mass
    from dcgrid_gb300 import DcgError, Simulation
    sim = Simulation(scenarios.ref_default(32, 32, 32, 120))
    sim.step(1)
    q = sim.get_field("density")
    q[_leaf_cell(sim) + 21] = np.nan
    sim.set_field("density", q)
    sim.step(1)
    with pytest.raises(DcgError) as e:
        sim.stats()
    assert e.value.code == capi.DCG_E_NAN
    with pytest.raises(DcgError) as e:
        sim.sync()
    assert e.value.code == capi.DCG_E_NAN


def test_nan_in_a_batch_member_is_reported():
    from dcgrid_gb300 import Batch, DcgError
    ps = [scenarios.plume(32, 64, 32, None, 2, 10), scenarios.plume(32, 32, 32, None, 2, 10)]
    b = Batch(ps)
    b.step(2)
    assert all(st.device_error == 0 for st in b.stats())
    m = b[1]
    p = m.get_field("pressure")
    p[_leaf_cell(m)] = np.inf
    m.set_field("pressure", p)
    with pytest.raises(DcgError) as e:
        b.stats()
    assert e.value.code == capi.DCG_E_NAN and "member 1" in str(e.value)
    with pytest.raises(DcgError) as e:
        b.sync()
    assert e.value.code == capi.DCG_E_NAN


def test_bounded_barrier_wait_gives_up_and_the_handle_recovers():
    from dcgrid_gb300 import Simulation
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    sim = Simulation(p)
    L = sim.L
    assert L.dcg_check_barrier_timeout(sim.h, 0) == capi.DCG_E_INVALID
    assert L.dcg_check_barrier_timeout(sim.h, 1000) == capi.DCG_OK
    assert L.dcg_sync(sim.h) == capi.DCG_E_DEVICE
    assert "bounded device-side wait" in L.dcg_last_error_string(sim.h).decode()
    rc, st = _stats_rc(sim)
    assert st.device_error & capi.DEVERR_TIMEOUT
    # the context is usable: after a reset the handle steps like a new one
    sim.reset()
    assert L.dcg_sync(sim.h) == capi.DCG_OK
    sim.add_velocity_noise(0, 0.01)
    sim.step(2)
    sim.sync()
    fresh = Simulation(p)
    fresh.add_velocity_noise(0, 0.01)
    fresh.step(2)
    for f in ["density", "vel_y", "pressure"]:
        assert np.array_equal(sim.get_field(f), fresh.get_field(f))
