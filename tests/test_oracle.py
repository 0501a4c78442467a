"""CPU tests of the oracle itself: the reference's budget split, error
behaviour, the incremental apron refresh against a fresh lookup, and
hand-checkable properties of each stage."""
import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

pytestmark = pytest.mark.usefixtures("oracle_lib")


def make(p, prec="double", mode=capi.MODE_ADAPTIVE):
    from oracle.pyoracle import OracleSim
    return OracleSim(p, mode=mode, precision=prec)


def alloc_cells(sim):
    t = sim.get_topology()
    return np.repeat(t["pos"][:, 3] >= 0, 64)


def test_budget_split_matches_reference_formula():
    # fluid_simulation_dcgrid.cu:29-69 for a 256^3 domain and a 40k budget
    p = scenarios.ref_default(256, 256, 256, 40000)
    p.init_adapt_passes = 0
    s = make(p)
    lv = s.info.levels
    assert lv == 7
    assert list(s.info.budget)[:lv] == [17660, 17659, 4096, 512, 64, 8, 1]
    assert list(s.info.full_blocks)[:lv] == [262144, 32768, 4096, 512, 64, 8, 1]
    assert s.info.sparse_levels == 2
    # 64x128x64 derives 5 levels (cu:16-22)
    p = scenarios.ref_default(64, 128, 64, 3000)
    p.init_adapt_passes = 0
    assert make(p).info.levels == 5


def test_errors_are_status_codes():
    from oracle.pyoracle import OracleError
    p = scenarios.ref_default(32, 64, 32, 1)  # fewer blocks than the coarsest level
    with pytest.raises(OracleError, match="DCG_E_BUDGET"):
        make(p)
    p = scenarios.ref_default(40, 64, 32, 600)
    p.levels = 4  # 40 is not a multiple of the coarsest block extent 32
    with pytest.raises(OracleError, match="DCG_E_INVALID"):
        make(p)
    p = scenarios.ref_default(32, 64, 32, 600)
    p.jacobi_iters = 3
    with pytest.raises(OracleError, match="DCG_E_INVALID"):
        make(p)


@pytest.mark.parametrize("name,compat", [("ref", 1), ("ref", 0), ("sphere", 1), ("cloud", 0), ("cloud", 1),
                                         ("plume", 1)])
def test_incremental_apron_equals_fresh_lookup(name, compat):
    """The reference refreshes apron entries incrementally after moves and
    refinements (dcgrid_structure.cu:30-92); the GPU path rebuilds neighbour
    tables from scratch. Both must give the same table."""
    p = {"ref": lambda: scenarios.ref_default(64, 64, 64, 1500),
         "sphere": lambda: scenarios.sphere_obstacle(64, 128, 64, 3000),
         "cloud": lambda: scenarios.cloud(64, 1500, 3, 10, compat),
         "plume": lambda: scenarios.plume(32, 64, 32, None, 2, 10)}[name]()
    p.ref_compat = compat
    s = make(p, "float")
    s.add_velocity_noise(3, 0.5)
    assert s.apron_mismatches() == 0
    moved = refined = 0
    for _ in range(6):
        s.step(1)
        st = s.stats()
        moved += st.moved_blocks
        refined += st.refined_subblocks
        assert s.apron_mismatches() == 0
    if name == "cloud":
        assert moved + refined > 0, "scenario should exercise topology changes"


def test_advection_with_zero_velocity_is_identity():
    p = scenarios.ref_default(32, 64, 32, 600)
    p.inlet_enabled = 0
    s = make(p, "float")
    m = alloc_cells(s)
    rng = np.random.default_rng(0)
    rho = rng.random(s.num_cells)
    s.set_field("density", rho.astype(np.float32).astype(np.float64))
    before = s.get_field("density")
    s.advect_scalars()
    after = s.get_field("density")
    t = s.get_topology()
    leaf = np.repeat((t["child"] == 0xFFFFFFFF).reshape(-1), 8) & m
    assert np.array_equal(after[leaf], before[leaf])


def test_restriction_is_mean_of_children():
    p = scenarios.plume(32, 64, 32, None, 2, 10)
    s = make(p, "float")
    s.add_velocity_noise(1, 1.0)
    s.step(1)
    rho = s.get_field("density")
    t = s.get_topology()
    pos, parent = t["pos"], t["parent"]
    checked = 0
    for b in np.nonzero(pos[:, 3] >= 0)[0]:
        if parent[b] == 0xFFFFFFFF:
            continue
        for sub in range(8):
            kids = rho[64 * b + 8 * sub: 64 * b + 8 * sub + 8].astype(np.float32)
            acc = np.float32(0)
            for k in kids:
                acc = np.float32(acc + k)
            assert np.float32(acc * np.float32(0.125)) == np.float32(rho[8 * int(parent[b]) + sub])
            checked += 1
    assert checked > 0


def test_projection_reduces_divergence():
    p = scenarios.plume(32, 64, 32, None, 2, 200)
    s = make(p)
    s.add_velocity_noise(5, 1.0)
    s.project()
    d0 = np.abs(s.get_field("divergence")).sum()
    s.project()
    d1 = np.abs(s.get_field("divergence")).sum()
    assert d1 < 0.9 * d0  # collocated central differences: partial reduction per projection


def test_float_mirror_close_to_fp64():
    p = scenarios.plume(32, 64, 32, None, 2, 20)
    a, b = make(p, "float"), make(p, "double")
    for s in (a, b):
        s.add_velocity_noise(0, 0.01)
        s.step(3)
    m = alloc_cells(a)
    for f in ["density", "temperature", "vel_y", "pressure"]:
        x, y = a.get_field(f)[m], b.get_field(f)[m]
        assert np.linalg.norm(x - y) <= 1e-4 * max(np.linalg.norm(y), 1e-12), f


def test_uniform_oracle_identity_and_mass():
    p = scenarios.plume(32, 64, 32, None, 0, 10)
    p.levels = 0
    s = make(p, "float", capi.MODE_UNIFORM)
    assert s.info.levels == 4
    s.step(2)
    st = s.stats()
    assert st.mass > 0
    rho = s.get_field("density")
    assert rho.max() <= 1.0 + 1e-6 and rho.min() >= -1e-6


def test_dense_resampling_covers_domain():
    p = scenarios.ref_default(32, 64, 32, 600)
    s = make(p)
    s.step(2)
    d = s.get_dense("density")
    assert d.shape == (32, 64, 32)
    assert np.isfinite(d).all()


def test_fp64_defect_correction_reduces_the_pressure_residual():
    """Defect correction (extension): each pass lowers the FP64 residual of the
    cascade's equations; no passes leaves the reference cascade unchanged."""
    from oracle.pyoracle import OracleSim
    base = scenarios.plume(32, 64, 32, None, 2, 10)
    rels = []
    p_fields = []
    for passes in (0, 1, 3):
        p = capi.params_from_dict(capi.params_to_dict(base))
        p.defect_passes = passes
        o = OracleSim(p, precision="double")
        o.add_velocity_noise(5, 0.5)
        o.step(2)
        st = o.stats()
        rels.append(tuple(st.defect_rel_residual))
        p_fields.append(o.get_field("pressure"))
    assert rels[0] == (0.0, 0.0)
    assert rels[1][1] < rels[1][0] and rels[2][1] < rels[1][1]
    assert not np.array_equal(p_fields[0], p_fields[2])
