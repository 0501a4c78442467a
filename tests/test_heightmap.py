"""Terrain from a heightmap (dcg_set_heightmap).

CPU (oracle): a constant map equals the flat noise terrain at the same
height, bit for bit, in the fields and in the rendered image; the map shapes
the solid (cells well below its lowest height are solid, well above its
highest are fluid, both kinds and partial cells occur); removing the map
returns to the noise terrain of a new handle; invalid shapes are refused.
GPU: the CUDA path against the oracle's float mirror, bit-exact, adaptive and
uniform, after the reset the call performs and after steps.
"""
import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

FIELDS = ["density", "vel_x", "vel_y", "vel_z", "fluidity", "pressure", "temperature"]


def orc(p, prec="float", mode=capi.MODE_ADAPTIVE):
    from oracle.pyoracle import OracleSim
    return OracleSim(p, mode=mode, precision=prec)


def terrain_cloud():
    """64^3 cloud scene on the heightmap: heights 4 + 20 * m cells."""
    p = scenarios.cloud(64, 1500, 3, 10, 0)
    p.terrain_base_height, p.terrain_amplitude = 4.0, 20.0
    return p


def same_fields(a, b, names=FIELDS):
    for f in names:
        x, y = a.get_field(f), b.get_field(f)
        assert np.array_equal(x, y), f"{f}: {(x != y).sum()} cells differ"


@pytest.mark.usefixtures("oracle_lib")
def test_constant_map_equals_flat_noise_terrain():
    p = terrain_cloud()
    p.terrain_base_height, p.terrain_amplitude = 10.0, 1.0
    a = orc(p)
    a.set_heightmap(np.full((5, 7), 5.0, np.float32))  # heights 10 + 1 * 5
    q = terrain_cloud()
    q.terrain_base_height, q.terrain_amplitude = 15.0, 0.0  # 15 + 0 * noise
    b = orc(q)
    same_fields(a, b)
    for s in (a, b):
        s.add_velocity_noise(3, 0.3)
        s.step(2)
    same_fields(a, b)


@pytest.mark.usefixtures("oracle_lib")
def test_map_shapes_the_solid():
    """Heights 12 + 20 m, m in [0, 1]. A leaf cell of edge s <= 4 (three
    levels) is solid when its SDF is <= -0.866 s and fluid when >= 0.866 s, so
    every finest row j <= 6 lies in a solid leaf cell and every row j >= 37 in
    a fluid one."""
    p = terrain_cloud()
    p.terrain_base_height, p.terrain_amplitude = 12.0, 20.0
    s = orc(p, "double")
    s.set_heightmap(scenarios.heightmap(48, 40, 1))
    w = s.get_dense("fluidity")  # (gz, gy, gx)
    assert (w[:, :7, :] == 0).all()
    assert (w[:, 37:, :] == 1).all()
    assert ((w > 0) & (w < 1)).any()
    rows = (w < 1).any(axis=(0, 2)).nonzero()[0]
    assert 12 <= rows.max() < 37  # the terrain's top follows the map, below 12 + 20 + margin


@pytest.mark.usefixtures("oracle_lib")
def test_removing_the_map_restores_the_noise_terrain():
    p = terrain_cloud()
    a, b = orc(p), orc(p)
    a.set_heightmap(scenarios.heightmap(48, 40, 2))
    assert not np.array_equal(a.get_field("fluidity"), b.get_field("fluidity"))
    a.set_heightmap(None)
    same_fields(a, b)


@pytest.mark.usefixtures("oracle_lib")
def test_renderer_sees_the_map():
    """The ray march shades the same SDF: a constant map renders exactly as
    the flat noise terrain at that height, a shaped map differently."""
    from tests.test_render_oracle import render_params
    p = terrain_cloud()
    p.terrain_base_height, p.terrain_amplitude = 10.0, 1.0
    flat_map = orc(p)
    flat_map.set_heightmap(np.full((5, 7), 5.0, np.float32))
    q = terrain_cloud()
    q.terrain_base_height, q.terrain_amplitude = 15.0, 0.0
    flat_noise = orc(q)
    rp = render_params(p, 32, 24, solids=1, shadows=1)
    a, b = flat_map.render(rp), flat_noise.render(rp)
    assert np.isfinite(a).all() and np.array_equal(a, b)
    hills = orc(terrain_cloud())
    hills.set_heightmap(scenarios.heightmap(48, 40, 1))
    assert not np.array_equal(hills.render(rp), b)


@pytest.mark.usefixtures("oracle_lib")
def test_invalid_maps_are_refused(dcg_lib):
    import ctypes as C
    from oracle.pyoracle import OracleError
    s = orc(terrain_cloud())
    with pytest.raises(OracleError):
        s.set_heightmap(np.zeros((0, 4), np.float32))
    one = np.zeros(1, np.float32)
    ptr = C.c_void_p(one.ctypes.data)
    assert s.L.dcgo_set_heightmap(s.h, None, 3, 3) == capi.DCG_E_INVALID  # sizes without heights
    assert s.L.dcgo_set_heightmap(s.h, ptr, 70000, 1) == capi.DCG_E_INVALID  # refused before any read
    assert dcg_lib.dcg_set_heightmap(None, None, 0, 0, capi.HOST) == capi.DCG_E_INVALID


def gpu(p, mode=capi.MODE_ADAPTIVE):
    from dcgrid_gb300 import Simulation
    return Simulation(p, mode)


@pytest.mark.gpu
@pytest.mark.usefixtures("cuda_ok", "dcg_lib", "oracle_lib")
def test_adaptive_heightmap_bitexact_vs_oracle():
    from tests.test_parity_gpu import compare
    p = terrain_cloud()
    hm = scenarios.heightmap(48, 40, 1)
    g, o = gpu(p), orc(p)
    for s in (g, o):
        s.set_heightmap(hm)
    g.sync()
    compare(g, o, p, "after set_heightmap")
    for s in (g, o):
        s.add_velocity_noise(4, 0.3)
    for k in range(3):
        for s in (g, o):
            s.step(1)
        g.sync()
        compare(g, o, p, f"step {k}")
    g.set_heightmap(None)
    o.set_heightmap(None)
    g.sync()
    compare(g, o, p, "noise terrain again")


@pytest.mark.gpu
@pytest.mark.usefixtures("cuda_ok", "dcg_lib", "oracle_lib")
def test_uniform_heightmap_bitexact_vs_oracle():
    p = scenarios.plume(32, 64, 32, None, 0, 10)
    p.levels = 0
    p.solids = capi.SOLIDS_TERRAIN
    p.terrain_base_height, p.terrain_amplitude = 2.0, 10.0
    hm = scenarios.heightmap(24, 20, 3)
    g, o = gpu(p, capi.MODE_UNIFORM), orc(p, "float", capi.MODE_UNIFORM)
    for s in (g, o):
        s.set_heightmap(hm)
        s.add_velocity_noise(9, 0.1)
        s.step(2)
    g.sync()
    for f in ["density", "temperature", "vel_x", "vel_y", "vel_z", "pressure", "fluidity"]:
        a, b = g.get_field(f), o.get_field(f).astype(np.float32)
        assert np.array_equal(a, b), f"{f}: {(a != b).sum()} cells differ"
