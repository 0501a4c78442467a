"""Known answers for the oracle's stages (FP64), from the mathematics of the
scheme rather than from another implementation.

* Semi-Lagrangian advection with trilinear sampling (dcgrid_fluid.cu:7-144,
  uniformgrid_fluid.cu) reproduces linear functions: a linear scalar carried
  by a uniform velocity is shifted exactly, f(x) -> f(x - v dt rdx), and a
  uniform velocity advects itself unchanged, away from the walls.
* The central-difference divergence (dcgrid_fluid.cu:174-230) of the linear
  field v = (a x, b y, c z) is rdx (a + b + c) in every interior cell.
* Refinement fills a new block by trilinear (27/9/3/1) prolongation from
  its parent's neighbourhood (dcgrid_adaptation.cu:92-143): exact for
  linear density and velocity.
* The leaf cells tile the domain exactly once at any level count, so
  sum_l leaf_cells[l] 8^l = gx gy gz, and the statistics' mass of a constant
  density (uniformgrid_structure.cu:41-42) is that density times the volume.

The adaptive cases that interpolate use one dense level, so no stencil meets
a level boundary (where the reference's ghost cells take the covering coarse
cell's value and linear functions are no longer reproduced).
"""
import numpy as np
import pytest

from dcgrid_gb300 import capi

pytestmark = pytest.mark.usefixtures("oracle_lib")

G = 32
MODES = [(capi.MODE_UNIFORM, 1), (capi.MODE_ADAPTIVE, 1)]
MODE_IDS = ["uniform", "adaptive_one_level"]


def params(levels, blocks=(G // 4) ** 3):
    p = capi.default_params(G, G, G, blocks)
    p.levels = levels
    p.dx, p.dt = 1.0, 1.0
    p.inlet_enabled = 0
    p.solids = capi.SOLIDS_NONE
    p.n_scalars = 1
    return p


def make(mode, levels, blocks=(G // 4) ** 3):
    from oracle.pyoracle import OracleSim
    return OracleSim(params(levels, blocks), mode=mode, precision="double")


def centres(s):
    """Finest-cell coordinates (n, 3) of every cell's centre in the canonical
    layout, and the mask of allocated cells."""
    if s.mode == capi.MODE_UNIFORM:
        z, y, x = np.meshgrid(np.arange(G), np.arange(G), np.arange(G), indexing="ij")
        return np.stack([x.ravel(), y.ravel(), z.ravel()], 1) + 0.5, np.ones(G ** 3, bool)
    pos = s.get_topology()["pos"]
    c = np.arange(64)
    sub = c >> 3
    local = np.stack([(((sub >> 2) & 1) << 1) | ((c >> 2) & 1),   # local order of dcgrid_utils.cuh:69-81
                      (((sub >> 1) & 1) << 1) | ((c >> 1) & 1),
                      ((sub & 1) << 1) | (c & 1)], 1)
    scale = (2.0 ** pos[:, 3])[:, None, None]
    X = (pos[:, None, :3] + local[None, :, :] + 0.5) * scale
    return X.reshape(-1, 3), np.repeat(pos[:, 3] >= 0, 64)


def interior(X, valid, margin):
    return valid & ((X >= margin) & (X <= G - margin)).all(axis=1)


@pytest.mark.parametrize("mode,levels", MODES, ids=MODE_IDS)
def test_linear_scalar_is_shifted_exactly(mode, levels):
    s = make(mode, levels)
    X, valid = centres(s)
    v = np.array([0.3, -0.2, 0.45])
    for k, f in enumerate(["vel_x", "vel_y", "vel_z"]):
        s.set_field(f, np.full(len(X), v[k]))
    grad = np.array([0.01, 0.02, -0.015])
    rho = 1.0 + X @ grad
    s.set_field("density", rho)
    s.advect_scalars()
    got = s.get_field("density")
    inner = interior(X, valid, 3)
    assert inner.sum() > 1000
    np.testing.assert_allclose(got[inner], (rho - grad @ v)[inner], rtol=0, atol=1e-12)


@pytest.mark.parametrize("mode,levels", MODES, ids=MODE_IDS)
def test_uniform_velocity_advects_itself_unchanged(mode, levels):
    s = make(mode, levels)
    X, valid = centres(s)
    v = [0.3, -0.2, 0.45]
    for k, f in enumerate(["vel_x", "vel_y", "vel_z"]):
        s.set_field(f, np.full(len(X), v[k]))
    s.advect_velocity()
    inner = interior(X, valid, 3)
    for k, f in enumerate(["vel_x", "vel_y", "vel_z"]):
        np.testing.assert_allclose(s.get_field(f)[inner], v[k], rtol=0, atol=1e-14, err_msg=f)


@pytest.mark.parametrize("mode,levels", MODES, ids=MODE_IDS)
def test_divergence_of_a_linear_field(mode, levels):
    s = make(mode, levels)
    X, valid = centres(s)
    a, b, c = 0.05, -0.02, 0.03
    s.set_field("vel_x", a * X[:, 0])
    s.set_field("vel_y", b * X[:, 1])
    s.set_field("vel_z", c * X[:, 2])
    s.project()
    inner = interior(X, valid, 2)
    rdx = 1.0 / s.params.dx
    np.testing.assert_allclose(s.get_field("divergence")[inner], rdx * (a + b + c), rtol=1e-12)


@pytest.mark.parametrize("levels,blocks", [(1, (G // 4) ** 3), (3, 8 + 64 + 128), (3, 8 + 32 + 40)])
def test_leaf_cells_tile_the_domain_and_mass_is_density_times_volume(levels, blocks):
    s = make(capi.MODE_ADAPTIVE, levels, blocks)
    s.set_field("density", np.full(s.num_cells, 0.25))
    st = s.stats()
    covered = sum(int(st.leaf_cells[l]) * 8 ** l for l in range(levels))
    assert covered == G ** 3
    assert st.mass == 0.25 * G ** 3
    u = make(capi.MODE_UNIFORM, 1)
    u.set_field("density", np.full(G ** 3, 0.25))
    assert u.stats().mass == 0.25 * G ** 3


def test_refinement_prolongs_linear_fields_exactly():
    """A replayed refinement of an interior subblock fills the new block by
    the 27/9/3/1 stencil from the parent's neighbourhood
    (dcgrid_adaptation.cu:92-143): trilinear interpolation at the child
    centres, exact for linear fields."""
    from oracle.pyoracle import OracleSim
    p = params(2, 64 + 64)
    p.init_adapt_passes = 0  # level 1 dense, level 0 empty: every leaf on level 1
    s = OracleSim(p, precision="double")
    assert list(s.get_topology()["load"]) == [0, 64]
    X, valid = centres(s)
    grads = {"density": [0.01, 0.02, -0.015], "vel_x": [0.3, -0.1, 0.05],
             "vel_y": [-0.02, 0.04, 0.01], "vel_z": [0.0, 0.07, -0.03]}
    for f, gvec in grads.items():
        s.set_field(f, 2.0 + X @ np.array(gvec))
    pos = s.get_topology()["pos"]
    pb = int(np.nonzero((pos == [4, 4, 4, 1]).all(axis=1))[0][0])  # level-1 block at finest 8..15
    s.adapt_replay(np.zeros((0, 2), np.int64), [(8 * pb + 7, 0)])  # its upper subblock -> block 0
    pos = s.get_topology()["pos"]
    assert list(pos[0]) == [12, 12, 12, 0]  # finest cells 12..15: every stencil inside the domain
    X, _ = centres(s)
    new = slice(0, 64)
    for f, gvec in grads.items():
        np.testing.assert_allclose(s.get_field(f)[new], (2.0 + X @ np.array(gvec))[new], rtol=0, atol=1e-12,
                                   err_msg=f)


def test_linear_shift_holds_for_random_velocities_and_gradients():
    """The exact shift of a linear scalar for random uniform velocities (up to
    0.9 cells per step in each direction) and random gradients."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    comp = st.floats(-0.9, 0.9, allow_nan=False)
    slope = st.floats(-0.05, 0.05, allow_nan=False)
    s = make(capi.MODE_UNIFORM, 1)
    X, valid = centres(s)
    inner = interior(X, valid, 3)

    @hyp.settings(max_examples=25, deadline=None, database=None)
    @hyp.given(st.tuples(comp, comp, comp), st.tuples(slope, slope, slope))
    def check(v, grad):
        v, grad = np.array(v), np.array(grad)
        for k, f in enumerate(["vel_x", "vel_y", "vel_z"]):
            s.set_field(f, np.full(len(X), v[k]))
        rho = 1.0 + X @ grad
        s.set_field("density", rho)
        s.advect_scalars()
        np.testing.assert_allclose(s.get_field("density")[inner], (rho - grad @ v)[inner], rtol=0, atol=1e-12)

    check()
