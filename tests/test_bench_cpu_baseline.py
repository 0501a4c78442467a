"""The benchmark's CPU baseline leg (bench.cpu_sample) on the CPU: the FP64
oracle started from a simulation's state, timed on all host threads and then
on one thread. Oracle simulations stand in for the GPU ones (the leg reads
only their block table and fields)."""
import os

import pytest

from tests import scenarios


@pytest.mark.usefixtures("oracle_lib")
def test_cpu_sample_reports_all_threads_and_one():
    import bench
    from oracle.pyoracle import OracleSim
    p = scenarios.plume(16, 32, 16, None, 2, 4)
    src = OracleSim(p, precision="double")
    src.add_velocity_noise(1, 0.1)
    src.step(1)
    out = bench.cpu_sample([src], [p], 1)
    assert out["kind"] == "port" and out["unit"] == bench.METRIC
    assert out["cores"] == (os.cpu_count() or 1) and out["value"] > 0
    one = out["single_core"]
    assert one["cores"] == 1 and one["value"] > 0 and one["unit"] == bench.METRIC
