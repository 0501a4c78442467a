"""FP64 host adjoint of the density path (oracle, CPU): dot-product tests.

With the flow and the topology held fixed the step maps the density and the
emission map affinely, so for perturbations dq, dE and any adjoint lam
  <lam, q_t(q + dq, E) - q_t(q, E)> = <J_q^T lam, dq>,
  <lam, q_t(q, E + dE) - q_t(q, E)> = <J_E^T lam, dE>,
and the dense resampling D satisfies <mu, D q> = <D^T mu, q>. Scenes use the
position-based refinement score (topology independent of the density) and no
buoyancy (flow independent of the density).
"""
import numpy as np
import pytest

from tests import scenarios


def orc(p):
    from oracle.pyoracle import OracleSim
    return OracleSim(p, precision="double")


def scene(g=32, levels=2):
    p = scenarios.differentiable(g, levels, iters=10, em_n=8, noise=0.5)
    return p


def spun_up(p, steps, em):
    o = orc(p)
    o.set_emission(em)
    o.add_velocity_noise(0, 0.5)
    o.step(steps)
    return o


def alloc_cells(o):
    return np.repeat(o.get_topology()["pos"][:, 3] >= 0, 64)


@pytest.mark.parametrize("levels", [2, 3])
def test_step_adjoint_is_the_transpose_in_density(levels):
    p = scene(32, levels)
    rng = np.random.default_rng(1)
    em = scenarios.emission_field(8, 3)
    base = spun_up(p, 3, em)
    a, b = orc(p), orc(p)
    a.copy_state_from(base)
    b.copy_state_from(base)
    cells = alloc_cells(base)
    dq = np.where(cells, rng.standard_normal(cells.size), 0.0)
    b.set_field("density", b.get_field("density") + dq)
    a.step(1)
    b.step(1)
    jdq = b.get_field("density") - a.get_field("density")
    lam = np.where(alloc_cells(a), rng.standard_normal(cells.size), 0.0)
    jt = a.adjoint_step(lam)
    st = a.stats()
    assert levels == 2 or st.moved_blocks + st.refined_subblocks > 0  # propagation transpose exercised
    lhs, rhs = float(lam @ jdq), float(jt @ dq)
    assert abs(lhs - rhs) <= 1e-9 * max(abs(lhs), 1.0), (lhs, rhs)


def test_step_adjoint_is_the_transpose_in_emission():
    p = scene(32, 2)
    rng = np.random.default_rng(2)
    em = scenarios.emission_field(8, 3).astype(np.float64)
    base = spun_up(p, 2, em)
    a, b = orc(p), orc(p)
    a.copy_state_from(base)
    b.copy_state_from(base)
    de = rng.standard_normal(em.size)
    b.set_emission(em + de)
    a.step(1)
    b.step(1)
    jde = b.get_field("density") - a.get_field("density")
    lam = np.where(alloc_cells(a), rng.standard_normal(jde.size), 0.0)
    lam_em = np.zeros(em.size)
    a.adjoint_step(lam, lam_em)
    lhs, rhs = float(lam @ jde), float(lam_em @ de)
    assert abs(lhs - rhs) <= 1e-9 * max(abs(lhs), 1.0), (lhs, rhs)


def test_adaptation_touches_blocks_in_the_checked_steps():
    """the dot tests above cover the propagation transpose only if blocks move
    or are created in the stepped state"""
    p = scene(32, 3)
    o = spun_up(p, 0, scenarios.emission_field(8, 3))
    moved = 0
    for _ in range(4):
        o.step(1)
        st = o.stats()
        moved += st.moved_blocks + st.refined_subblocks
    assert moved > 0


def test_dense_adjoint_is_the_transpose():
    p = scene(32, 3)
    rng = np.random.default_rng(3)
    o = spun_up(p, 2, scenarios.emission_field(8, 3))
    q = np.where(alloc_cells(o), rng.standard_normal(64 * p.max_blocks), 0.0)
    o.set_field("density", q)
    dense = o.get_dense("density").reshape(-1)
    mu = rng.standard_normal(dense.size)
    lam = np.zeros(q.size)
    o.adjoint_dense(mu, lam)
    lhs, rhs = float(mu @ dense), float(lam @ q)
    assert abs(lhs - rhs) <= 1e-9 * max(abs(lhs), 1.0), (lhs, rhs)
