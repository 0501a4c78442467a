"""dcg_get_dense_noalloc: the dense read-out for callers that cannot allocate
device memory when they read (during stream capture, under a fixed memory
budget, in loops that must not wait on the allocator). It must give exactly
what dcg_get_dense gives, call after call, through the C ABI.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib")]


def bind(L):
    L.dcg_get_dense_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]
    L.dcg_get_dense_noalloc.restype = C.c_int
    return L


def noalloc_dense(sim, field):
    L = bind(sim.L)
    p = sim.params
    out = np.full(p.gx * p.gy * p.gz, np.nan, np.float32)
    rc = L.dcg_get_dense_noalloc(sim.h, capi.FIELD_NAMES[field], C.c_void_p(out.ctypes.data), capi.HOST)
    assert rc == capi.DCG_OK, sim.L.dcg_last_error_string(sim.h).decode()
    return out.reshape(p.gz, p.gy, p.gx)


def test_noalloc_matches_get_dense_on_two_calls_in_a_row():
    from dcgrid_gb300 import Simulation
    p = scenarios.cloud(64, 1500, 3, 10, 0)
    sim = Simulation(p)
    sim.add_velocity_noise(5, 0.5)
    sim.step(3)
    # two calls in a row, on different fields, each against dcg_get_dense
    a1 = noalloc_dense(sim, "density")
    a2 = noalloc_dense(sim, "vel_y")
    b1 = sim.get_dense("density")
    b2 = sim.get_dense("vel_y")
    assert np.array_equal(a1, b1)
    assert np.array_equal(a2, b2)
    assert not np.array_equal(a1, a2)
    # and again after the state has moved on
    sim.step(2)
    assert np.array_equal(noalloc_dense(sim, "temperature"), sim.get_dense("temperature"))
    assert np.array_equal(noalloc_dense(sim, "density"), sim.get_dense("density"))


def test_noalloc_device_destination():
    import torch
    from dcgrid_gb300 import Simulation
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    sim = Simulation(p)
    sim.step(2)
    L = bind(sim.L)
    t = torch.empty(32 * 64 * 32, dtype=torch.float32, device="cuda")
    rc = L.dcg_get_dense_noalloc(sim.h, capi.FIELD_DENSITY, C.c_void_p(t.data_ptr()), capi.DEVICE)
    assert rc == capi.DCG_OK
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy().reshape(32, 64, 32), sim.get_dense("density"))


def test_noalloc_rejects_volumes_beyond_its_scratch():
    from dcgrid_gb300 import Simulation
    p = scenarios.ref_default(128, 128, 128, 2000)
    p.levels = 3
    p.init_adapt_passes = 0
    sim = Simulation(p)
    L = bind(sim.L)
    out = np.empty(128 ** 3, np.float32)
    rc = L.dcg_get_dense_noalloc(sim.h, capi.FIELD_DENSITY, C.c_void_p(out.ctypes.data), capi.HOST)
    assert rc == capi.DCG_E_INVALID
    assert "exceeds" in sim.L.dcg_last_error_string(sim.h).decode()
