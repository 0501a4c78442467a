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


def test_buoyant_rollout_adjoint_matches_fp64_central_differences():
    """A buoyant rollout (temperature source, alpha = 0.1, beta = 0.3, an
    emission map): the gradient of a dense density loss with respect to the
    emission map through 8 steps of the full FP64 host adjoint equals FP64
    central differences along unit directions. In FP64 a step of 1e-6 along a
    unit direction moves no sample across a cell face or a level interface
    (where the semi-Lagrangian sample is not differentiable)."""
    from oracle.pyoracle import OracleSim
    g, steps, em_n = 32, 8, 8
    p = scenarios.differentiable(g, 2, iters=20, em_n=em_n)
    p.n_scalars = 3
    p.buoy_alpha, p.buoy_beta = 0.1, 0.3
    p.src_enabled = 1
    p.src_center[0], p.src_center[1], p.src_center[2] = g / 2.0, g / 8.0, g / 2.0
    p.src_radius = 3.0
    p.src_density, p.src_temperature, p.src_vapor = 0.0, 10.0, 0.0
    rng = np.random.default_rng(2)
    E0 = 0.05 * rng.random(em_n ** 3)
    base = OracleSim(p, precision="double")
    base.add_velocity_noise(0, 0.5)
    probe = _clone(base, p)
    probe.set_emission(E0)
    decisions = []
    for _ in range(steps):
        probe.advect_velocity()
        probe.adapt()
        decisions.append(probe.get_last_adapt())
        probe.project()
        probe.advect_scalars()
    target = 0.5 * probe.get_dense("density").reshape(-1)

    def run(E):
        o = _clone(base, p)
        o.set_emission(E)
        states = []
        for t in range(steps):
            states.append(_clone(o, p))
            _step(o, *decisions[t])
        return o, states

    def loss(E):
        o, _ = run(E)
        r = o.get_dense("density").reshape(-1) - target
        return float(r @ r)

    o, states = run(E0)
    nq, nc = p.n_scalars, o.num_cells
    lam = np.zeros((3 + nq) * nc)
    lrho = np.zeros(nc)
    o.adjoint_dense(2.0 * (o.get_dense("density").reshape(-1) - target), lrho)
    lam[3 * nc:4 * nc] = lrho
    lam_e = np.zeros(em_n ** 3)
    for t in range(steps - 1, -1, -1):
        mv, rf = decisions[t]
        lam = states[t].adjoint_step_full(lam, lam_e, moves=mv, refines=rf)
    eps = 1e-6
    for _ in range(4):
        d = rng.standard_normal(em_n ** 3)
        d /= np.linalg.norm(d)
        fd = (loss(E0 + eps * d) - loss(E0 - eps * d)) / (2 * eps)
        an = float(lam_e @ d)
        assert abs(fd - an) <= 1e-5 * abs(fd), (fd, an)
