"""Memory-budget calculators (CPU): this layout's exact plan and the
reference's own estimates (scripts/calcMemory*.js, calcActiveBlocks.js)."""
import pytest

from dcgrid_gb300 import capi, memory, scenes


def test_reference_estimates_match_their_scripts():
    total, per_block = memory.reference_adaptive_bytes(1, 12)
    assert per_block == 5142  # the script's 12-channel per-block figure
    assert total == 96 + 5142
    # 64^3 uniform grid, 18 channels: 73 B per cell plus the coarser mips
    u = memory.reference_uniform_bytes(64, 64, 64)
    assert u == 64 ** 3 * 73 + (sum((64 // s) ** 3 for s in (1, 2, 4, 8, 16, 32, 64)) - 64 ** 3) * 4
    assert memory.reference_active_cells(10) == (71, 568)


def test_plan_grows_with_the_budget_and_formats():
    p = scenes.cloud256()
    a = memory.plan_bytes(p)
    p.max_blocks *= 2
    b = memory.plan_bytes(p)
    assert b > a
    p.precision = capi.PRECISION_MIXED_FP16
    assert memory.plan_bytes(p) < b  # 16-bit scalars


def test_blocks_for_budget_is_the_largest_that_fits():
    p = capi.default_params(256, 256, 256, 1)
    p.levels, p.n_scalars = 3, 3
    budget = 300 * 2 ** 20
    n = memory.blocks_for_budget(p, budget)
    p.max_blocks = n
    assert memory.plan_bytes(p) <= budget
    p.max_blocks = n + 1
    assert memory.plan_bytes(p) > budget


def test_blocks_for_budget_caps_at_full_coverage_and_rejects_tiny_budgets():
    p = capi.default_params(512, 512, 512, 1)
    p.levels, p.n_scalars = 4, 3
    full = sum((512 >> (2 + l)) ** 3 for l in range(4))
    assert memory.blocks_for_budget(p, 100 * 10 ** 9) == full
    with pytest.raises(Exception):
        memory.blocks_for_budget(p, 10 ** 6)


def test_uniform_edge_for_budget():
    p = capi.default_params(64, 64, 64, 1)
    p.n_scalars = 3
    e = memory.uniform_edge_for_budget(p, 10 * 10 ** 9)
    q = capi.params_from_dict(capi.params_to_dict(p))
    q.gx = q.gy = q.gz = e
    assert memory.plan_bytes(q, capi.MODE_UNIFORM) <= 10 * 10 ** 9
    q.gx = q.gy = q.gz = e + 64
    assert memory.plan_bytes(q, capi.MODE_UNIFORM) > 10 * 10 ** 9


@pytest.mark.gpu
@pytest.mark.usefixtures("cuda_ok", "dcg_lib")
@pytest.mark.parametrize("mode,prec,em", [(capi.MODE_ADAPTIVE, capi.PRECISION_FP32, 0),
                                          (capi.MODE_ADAPTIVE, capi.PRECISION_MIXED_FP16, 16),
                                          (capi.MODE_UNIFORM, capi.PRECISION_FP32, 8)])
def test_plan_equals_the_allocation(mode, prec, em):
    from dcgrid_gb300 import Simulation
    p = scenes.cloud(64, 1500, 3, 10, 0)
    p.precision, p.emission_n, p.emission_band = prec, em, 16.0
    s = Simulation(p, mode)
    assert s.info.device_bytes == memory.plan_bytes(p, mode)
