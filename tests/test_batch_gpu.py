"""Batched simulations (dcg_batch_*): many independent adaptive simulations per
launch must give every member exactly the results of a standalone simulation
with the same parameters, whatever the tuning, group split or precision."""
import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios
from tests.test_parity_gpu import compare, orc

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib")]


def small_batch(n=5, seed=3, precision=capi.PRECISION_FP32, iters=20):
    return scenarios.plume_batch(n, seed, sizes=(16, 32, 48, 64), iters=iters, precision=precision)


def standalone(p, steps):
    from dcgrid_gb300 import Simulation
    s = Simulation(p)
    s.add_velocity_noise(11, 0.05)
    s.step(steps)
    s.sync()
    return s


def batch_run(params, steps, tuning=None):
    from dcgrid_gb300 import Batch
    b = Batch(params)
    if tuning is not None:
        b.set_tuning(tuning)
    for m in b:
        m.add_velocity_noise(11, 0.05)
    b.step(steps)
    b.sync()
    return b


@pytest.mark.parametrize("prec", [capi.PRECISION_FP32, capi.PRECISION_MIXED_FP16, capi.PRECISION_MIXED],
                         ids=["fp32", "fp16", "bf16"])
def test_batch_members_equal_standalone(prec):
    params = small_batch(5, 3, prec)
    assert len({(p.gx, p.levels) for p in params}) > 1  # uneven members
    b = batch_run(params, 6)
    for i, p in enumerate(params):
        compare(b[i], standalone(p, 6), p, f"member {i}")


@pytest.mark.parametrize("staged", [False, True], ids=["tiled", "staged"])
def test_batch_mixed_precisions_and_levels_in_one_batch(staged):
    params = small_batch(5, 5)
    params[1].precision = capi.PRECISION_MIXED_FP16
    params[2].precision = capi.PRECISION_MIXED
    params[3].levels = 3 if params[3].levels == 2 else 2
    params[4].n_scalars = 1  # density only: another scalar-advection kernel
    params[4].precision = capi.PRECISION_MIXED_FP16
    b = batch_run(params, 4, tuning(1, 4, 0, 1, 1) if staged else None)
    for i, p in enumerate(params):
        compare(b[i], standalone(p, 4), p, f"member {i}")


def test_batch_member_equals_oracle():
    params = small_batch(3, 8)
    b = batch_run(params, 3)
    for i, p in enumerate(params):
        o = orc(p)
        o.add_velocity_noise(11, 0.05)
        o.step(3)
        compare(b[i], o, p, f"member {i} vs oracle")


def tuning(tile, cache, ctas, barrier, persistent=0):
    t = capi.DcgTuning()
    for k in range(4):
        t.tile[k] = tile
    t.solve_cache, t.solve_ctas_per_sm, t.solve_barrier = cache, ctas, barrier
    t.persistent = persistent
    return t


def test_results_do_not_depend_on_tuning():
    params = small_batch(5, 13)
    ref = batch_run(params, 5, tuning(4, 4, 0, 1))
    rounds = tuning(4, 4, 0, 1, 1)
    rounds.round_ctas_per_sm[0], rounds.round_cache[0], rounds.round_barrier[0] = 1, 0, 1
    rounds.round_ctas_per_sm[1], rounds.round_cache[1], rounds.round_barrier[1] = 2, 3, 0
    staged = tuning(1, 4, 0, 1, 1)
    # one CTA per SM makes the levels large enough for the staged sweeps;
    # variants 16 / 32 read block descriptions from the global table
    piped2, piped3 = tuning(4, 18, 1, 0, 1), tuning(1, 35, 1, 1, 1)
    piped_global2, piped_global3 = tuning(4, 16, 1, 1, 1), tuning(2, 32, 2, 0, 0)
    piped_rounds = tuning(4, 4, 0, 1, 1)
    piped_rounds.round_ctas_per_sm[1], piped_rounds.round_cache[1], piped_rounds.round_barrier[1] = 2, 34, 0
    piped_rounds.round_ctas_per_sm[0], piped_rounds.round_cache[0], piped_rounds.round_barrier[0] = -4, 18, 1
    mixed_tiles = tuning(4, 4, 0, 1, 0)
    mixed_tiles.tile[0], mixed_tiles.tile[3] = 1, 1
    for t in [tuning(2, 0, 1, 0), tuning(8, 8, 2, 1, 1), tuning(2, 8, 1, 0, 1), tuning(8, 0, 0, 1),
              tuning(4, 3, 0, 0, 1), rounds, staged, mixed_tiles, piped2, piped3, piped_rounds, piped_global2,
              piped_global3, tuning(1, 19, 0, 2, 1), tuning(2, 16, 1, 3, 1), tuning(1, 66, 1, 2, 1),
              tuning(1, 64, 1, 1, 1), tuning(1, 19, 1, 4, 1), tuning(4, 16, 2, 5, 1), tuning(1, 83, 1, 0, 1)]:
        b = batch_run(params, 5, t)
        for i, p in enumerate(params):
            compare(b[i], ref[i], p, f"tiles {list(t.tile)} cache {t.solve_cache} member {i}")


def test_groups_beyond_sixteen_members():
    params = scenarios.plume_batch(18, 21, sizes=(16, 32), iters=10)
    b = batch_run(params, 3)
    for i in [0, 7, 15, 16, 17]:
        compare(b[i], standalone(params[i], 3), params[i], f"member {i}")


def test_autotune_resets_and_keeps_results():
    from dcgrid_gb300 import Batch
    params = small_batch(4, 17)
    b = Batch(params)
    t = b.autotune(spinup_steps=3, reps=2)
    assert all(x in (1, 2, 4, 8) for x in t["tile"])
    assert t["solve_cache"] in (0, 3, 4, 8, 16, 18, 19, 32, 34, 35, 64, 66, 83) and 0 <= t["solve_barrier"] <= 7
    assert t["solve_ms"] > 0
    fresh = Batch(params)
    for i, p in enumerate(params):
        compare(b[i], fresh[i], p, f"after autotune member {i}")
    for s in (b, fresh):
        for m in s:
            m.add_velocity_noise(11, 0.05)
        s.step(4)
        s.sync()
    for i, p in enumerate(params):
        compare(b[i], fresh[i], p, f"tuned vs default member {i}")
    info = b.info()
    assert info["n"] == 4 and info["launches_per_step"] > 0


def test_member_handles_are_borrowed():
    from dcgrid_gb300 import Batch, DcgError
    b = Batch(small_batch(2, 1))
    with pytest.raises(DcgError) as e:
        b[0].step(1)
    assert e.value.code == capi.DCG_E_INVALID
    with pytest.raises(DcgError):
        b[1].reset()
    assert b.L.dcg_destroy(b[0].h) == capi.DCG_E_INVALID
    b.step(1)
    b.sync()
    assert np.isfinite(b[0].get_field("density")).all()


@pytest.mark.parametrize("prec", [capi.PRECISION_FP32, capi.PRECISION_MIXED_FP16], ids=["fp32", "fp16"])
def test_batch_defect_correction_members_equal_standalone(prec):
    """FP64 defect correction inside a batch: every member equals a standalone
    simulation with the same passes bit for bit (fields and topology); the
    relative residuals are FP64 sums of the same terms in another order."""
    params = small_batch(5, 23, prec)
    for q in params:
        q.defect_passes = 2
    b = batch_run(params, 4)
    bst = b.stats()
    for i, p in enumerate(params):
        s = standalone(p, 4)
        compare(b[i], s, p, f"member {i}")
        one = s.stats()
        assert one.defect_rel_residual[1] < one.defect_rel_residual[0]
        for k in range(2):
            assert bst[i].defect_rel_residual[k] == pytest.approx(one.defect_rel_residual[k], rel=1e-9)


def test_batch_defect_correction_member_equals_oracle():
    params = small_batch(3, 29)
    for q in params:
        q.defect_passes = 1
    b = batch_run(params, 3, tuning(1, 19, 0, 2, 1))
    for i, p in enumerate(params):
        o = orc(p)
        o.add_velocity_noise(11, 0.05)
        o.step(3)
        compare(b[i], o, p, f"member {i} vs oracle")


def test_batch_rejects_mixed_defect_passes():
    from dcgrid_gb300 import Batch, DcgError
    params = small_batch(2, 1)
    params[1].defect_passes = 1
    with pytest.raises(DcgError) as e:
        Batch(params)
    assert e.value.code == capi.DCG_E_INVALID


def test_batch_rejects_mixed_sweep_counts():
    from dcgrid_gb300 import Batch, DcgError
    params = small_batch(2, 1)
    params[1].jacobi_iters = params[0].jacobi_iters + 2
    with pytest.raises(DcgError) as e:
        Batch(params)
    assert e.value.code == capi.DCG_E_INVALID


def test_time_solve_reports_bytes():
    params = small_batch(3, 2)
    b = batch_run(params, 2)
    ms, nbytes = b.time_solve(3)
    assert ms > 0 and nbytes > 0


@pytest.mark.parametrize("persistent", [0, 1])
def test_batch_stats_equal_member_stats(persistent):
    params = small_batch(4, 6)
    b = batch_run(params, 3, tuning(4, 4, 0, 1, persistent))
    for st, m in zip(b.stats(), b):
        one = m.stats()
        assert st.active_cells == one.active_cells and list(st.load) == list(one.load)
        assert st.mass == pytest.approx(one.mass, rel=1e-12) and st.residual == pytest.approx(one.residual, rel=1e-9)


def test_headline_batch_full_size_members_equal_standalone():
    """The benchmark's workload at its full size (16 plumes of 64^3 to 256^3,
    2 or 3 levels, 100 sweeps per level, FP16 scalar storage, a 16^3 emission
    map each): after 4 steps every member equals the same plume stepped as a
    standalone simulation, bit for bit. A size-independent check at a size
    where the oracle would take minutes; the members' parity with the oracle
    is checked on small batches above."""
    from dcgrid_gb300 import Batch, Simulation
    params = scenarios.plume_batch(16, 0, sizes=(64, 96, 128, 192, 256), iters=100,
                                   precision=capi.PRECISION_MIXED_FP16, em_n=16)
    ems = [scenarios.emission_field(16, 100 + i) for i in range(16)]
    b = Batch(params)
    for i, m in enumerate(b):
        m.set_emission(ems[i])
        m.add_velocity_noise(11, 0.05)
    b.step(4)
    b.sync()
    for i, p in enumerate(params):
        s = Simulation(p)
        s.set_emission(ems[i])
        s.add_velocity_noise(11, 0.05)
        s.step(4)
        s.sync()
        compare(b[i], s, p, f"member {i} ({p.gx}^3, {p.levels} levels)")
        s.close()
    b.close()


def test_batch_emission_upload_equals_member_uploads():
    from dcgrid_gb300 import Batch
    params = scenarios.plume_batch(3, 4, sizes=(16, 32), iters=10, em_n=8)
    rng = np.random.default_rng(5)
    maps = [rng.random((8, 8, 8), dtype=np.float32) for _ in params]
    a, b = Batch(params), Batch(params)
    for i, m in enumerate(a):
        m.set_emission(maps[i])
    b.set_emission(np.concatenate([x.ravel() for x in maps]))
    for s in (a, b):
        s.step(3)
        s.sync()
    for i, p in enumerate(params):
        compare(a[i], b[i], p, f"member {i}")
