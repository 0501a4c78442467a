"""The FP64 host adjoint of one whole step (oracle, CPU): velocity and
scalars, buoyancy, the transposed pressure cascade and the dependence of the
semi-Lagrangian sample positions on the velocity. Checked against central
differences of the FP64 step itself, <lam, (F(x + e d) - F(x - e d)) / 2e> =
<F'^T lam, d>, with the adaptation decisions replayed so the topology is the
recorded one."""
import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

pytestmark = pytest.mark.usefixtures("oracle_lib")

STATE = ["vel_x", "vel_y", "vel_z", "density", "temperature", "vapor"]


def _clone(o, p):
    from oracle.pyoracle import OracleSim
    c = OracleSim(p, precision="double")
    c.copy_state_from(o)
    return c


def _state(o, nq):
    return np.concatenate([o.get_field(f) for f in STATE[:3 + nq]])


def _set_state(o, x, nq, nc):
    for i, f in enumerate(STATE[:3 + nq]):
        o.set_field(f, x[i * nc:(i + 1) * nc])


def _step(o, mv, rf):
    o.advect_velocity()
    o.adapt_replay(mv, rf)
    o.project()
    o.advect_scalars()


@pytest.mark.parametrize("compat", [0, 1])
def test_full_step_adjoint_matches_central_differences(compat):
    from oracle.pyoracle import OracleSim
    p = scenarios.plume(16, 32, 16, None, 2, 10)
    p.ref_compat = compat
    p.dt = 0.5
    o = OracleSim(p, precision="double")
    o.add_velocity_noise(3, 0.5)
    o.step(3)
    nq, nc = p.n_scalars, o.num_cells
    probe = _clone(o, p)
    probe.step(1)
    mv, rf = probe.get_last_adapt()
    rng = np.random.default_rng(7)
    alloc = np.repeat(o.get_topology()["pos"][:, 3] >= 0, 64)
    mask = np.tile(alloc, 3 + nq)
    lam = rng.standard_normal((3 + nq) * nc) * mask
    d = rng.standard_normal((3 + nq) * nc) * mask
    adj = _clone(o, p).adjoint_step_full(lam, moves=mv, refines=rf)
    x = _state(o, nq)
    eps = 1e-6
    ys = []
    for sgn in (1, -1):
        c = _clone(o, p)
        _set_state(c, x + sgn * eps * d, nq, nc)
        _step(c, mv, rf)
        ys.append(_state(c, nq))
    fd = float(np.dot(lam, (ys[0] - ys[1]) / (2 * eps)))
    an = float(np.dot(adj, d))
    assert abs(fd - an) <= 1e-6 * max(abs(fd), 1.0), (fd, an)


def test_full_step_adjoint_through_moves_and_refinements():
    """A step of the small cloud scene (wind inflow, field-driven refinement,
    buoyancy, sources) in which blocks move and new blocks are refined: the
    propagation transposes and the boundary pass-through rules of the wind.
    Without the terrain: cells inside a solid keep velocity components of
    exactly zero, so their back-traced samples sit on cell faces, where the
    trilinear interpolation has a kink; there the adjoint takes the derivative
    inside the cell the step samples and central differences average the two
    sides."""
    from oracle.pyoracle import OracleSim
    p = scenarios.cloud(32, 300, 2, 10, 0)
    p.solids = capi.SOLIDS_NONE
    o = OracleSim(p, precision="double")
    o.add_velocity_noise(3, 0.5)
    o.step(2)
    nq, nc = p.n_scalars, o.num_cells
    probe = _clone(o, p)
    probe.step(1)
    mv, rf = probe.get_last_adapt()
    assert len(mv) > 0 and len(rf) > 0
    rng = np.random.default_rng(5)
    alloc = np.repeat(o.get_topology()["pos"][:, 3] >= 0, 64)
    mask = np.tile(alloc, 3 + nq)
    lam = rng.standard_normal((3 + nq) * nc) * mask
    d = rng.standard_normal((3 + nq) * nc) * mask
    adj = _clone(o, p).adjoint_step_full(lam, moves=mv, refines=rf)
    x = _state(o, nq)
    eps = 1e-6
    ys = []
    for sgn in (1, -1):
        c = _clone(o, p)
        _set_state(c, x + sgn * eps * d, nq, nc)
        _step(c, mv, rf)
        ys.append(_state(c, nq))
    fd = float(np.dot(lam, (ys[0] - ys[1]) / (2 * eps)))
    an = float(np.dot(adj, d))
    assert abs(fd - an) <= 1e-6 * max(abs(fd), 1.0), (fd, an)


def test_full_step_adjoint_of_the_pressure_path_alone():
    """With the velocity adjoint only on v (no scalar adjoint) the answer is
    the projection and velocity advection path; a direction on the scalars
    alone then probes the buoyancy coupling into the velocity."""
    from oracle.pyoracle import OracleSim
    p = scenarios.plume(16, 32, 16, None, 2, 10)
    p.ref_compat = 0
    o = OracleSim(p, precision="double")
    o.add_velocity_noise(4, 0.3)
    o.step(2)
    nq, nc = p.n_scalars, o.num_cells
    probe = _clone(o, p)
    probe.step(1)
    mv, rf = probe.get_last_adapt()
    rng = np.random.default_rng(11)
    alloc = np.repeat(o.get_topology()["pos"][:, 3] >= 0, 64)
    lam = np.concatenate([rng.standard_normal(3 * nc) * np.tile(alloc, 3), np.zeros(nq * nc)])
    d = np.concatenate([np.zeros(3 * nc), rng.standard_normal(nq * nc) * np.tile(alloc, nq)])
    adj = _clone(o, p).adjoint_step_full(lam, moves=mv, refines=rf)
    x = _state(o, nq)
    eps = 1e-6
    ys = []
    for sgn in (1, -1):
        c = _clone(o, p)
        _set_state(c, x + sgn * eps * d, nq, nc)
        _step(c, mv, rf)
        ys.append(_state(c, nq))
    fd = float(np.dot(lam, (ys[0] - ys[1]) / (2 * eps)))
    an = float(np.dot(adj, d))
    assert abs(fd) > 1e-8  # buoyancy couples the scalars into the velocity
    assert abs(fd - an) <= 1e-6 * max(abs(fd), 1.0), (fd, an)
