"""dcg_get_dense_noalloc: the dense read-out for hosts that cannot let the
library allocate device memory when they read a field — hosts that hand it a
fixed device-memory budget up front, and frame loops that must not take
cudaMalloc's device-wide synchronisation. It must give exactly what
dcg_get_dense gives, call after call, through the C ABI (the Python wrapper
Simulation.get_dense_noalloc only checks the buffer and calls the entry
point).

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib")]


def test_noalloc_matches_get_dense_on_two_calls_in_a_row():
    from dcgrid_gb300 import Simulation
    p = scenarios.cloud(64, 1500, 3, 10, 0)
    sim = Simulation(p)
    sim.add_velocity_noise(5, 0.5)
    sim.step(3)
    # two calls in a row, on different fields, each against dcg_get_dense
    a1 = sim.get_dense_noalloc("density")
    a2 = sim.get_dense_noalloc("vel_y")
    b1 = sim.get_dense("density")
    b2 = sim.get_dense("vel_y")
    assert np.array_equal(a1, b1)
    assert np.array_equal(a2, b2)
    assert not np.array_equal(a1, a2)
    # and again after the state has moved on: the shared scratch keeps the
    # previous call's contents, which must not leak into the next result
    sim.step(2)
    assert np.array_equal(sim.get_dense_noalloc("temperature"), sim.get_dense("temperature"))
    assert np.array_equal(sim.get_dense_noalloc("density"), sim.get_dense("density"))


def test_noalloc_raw_c_abi_and_device_destination():
    import torch
    from dcgrid_gb300 import Simulation
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    sim = Simulation(p)
    sim.step(2)
    n = 32 * 64 * 32
    # the bare C entry point, host destination
    out = np.full(n, np.nan, np.float32)
    rc = sim.L.dcg_get_dense_noalloc(sim.h, capi.FIELD_DENSITY, C.c_void_p(out.ctypes.data), capi.HOST)
    assert rc == capi.DCG_OK, sim.L.dcg_last_error_string(sim.h).decode()
    ref = sim.get_dense("density")
    assert np.array_equal(out.reshape(32, 64, 32), ref)
    # device destination, through the wrapper
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    sim.get_dense_noalloc("density", out=t)
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy().reshape(32, 64, 32), ref)


def test_noalloc_rejects_volumes_beyond_its_scratch():
    from dcgrid_gb300 import DcgError, Simulation
    p = scenarios.ref_default(128, 128, 128, 2000)
    p.levels = 3
    p.init_adapt_passes = 0
    sim = Simulation(p)
    with pytest.raises(DcgError) as e:
        sim.get_dense_noalloc("density")
    assert e.value.code == capi.DCG_E_INVALID
    assert "exceeds" in str(e.value)
