"""CPU checks of the Python host layer (dcgrid_gb300/sim.py) against a fake C
library that records its calls: buffers of the wrong size, dtype, layout or
location are refused before the library is called (it would read or write
that many bytes behind the pointer), and the reference-named classes map the
reference's render(dest, resolution, eyePos, eyeDir, fov, sunDir) onto
dcg_render. No GPU and no compute calls."""
import ctypes as C

import numpy as np
import pytest

from dcgrid_gb300 import capi


class FakeLib:
    """Every dcg_* function returns DCG_OK and records (name, args);
    dcg_state_bytes reports STATE bytes."""
    STATE = 1000

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        if not name.startswith("dcg_"):
            raise AttributeError(name)

        def fn(*args):
            self.calls.append((name, args))
            if name == "dcg_state_bytes":
                args[1]._obj.value = self.STATE
            if name.endswith("last_error_string"):
                return b"fake"
            return capi.DCG_OK
        return fn

    def names(self):
        return [n for n, _ in self.calls]


def fake_sim(cls=None, blocks=100, emission_n=4):
    from dcgrid_gb300 import sim
    s = object.__new__(cls or sim.Simulation)
    s.L = FakeLib()
    s.h = C.c_void_p(1)
    s.params = capi.default_params(16, 32, 16, blocks)
    s.params.emission_n = emission_n
    s.mode = capi.MODE_ADAPTIVE
    s.info = capi.DcgInfo()
    s.info.max_blocks = blocks
    s.info.num_cells = 64 * blocks
    s.info.levels = 2
    return s


def refused(fn, *a, **k):
    from dcgrid_gb300 import DcgError
    with pytest.raises(DcgError) as e:
        fn(*a, **k)
    assert e.value.code == capi.DCG_E_INVALID
    return str(e.value)


def test_field_buffers_are_checked():
    s = fake_sim()
    n = s.num_cells
    refused(s.get_field, "density", np.empty(n - 1, np.float32))
    refused(s.get_field, "density", np.empty(n, np.float64))
    refused(s.get_field, "density", np.empty((2, n), np.float32)[:, 0])  # strided
    ro = np.empty(n, np.float32)
    ro.flags.writeable = False
    refused(s.get_field, "density", ro)
    refused(s.set_field, "density", np.zeros(n + 1))
    assert "dcg_get_field" not in s.L.names() and "dcg_set_field" not in s.L.names()
    out = s.get_field("density")
    assert out.shape == (n,) and out.dtype == np.float32
    s.set_field("density", np.zeros(n))  # converted to float32
    assert s.L.names() == ["dcg_get_field", "dcg_set_field"]


def test_emission_maps_are_checked():
    s = fake_sim(emission_n=4)
    msg = refused(s.set_emission, np.zeros(63, np.float32))
    assert "64 elements" in msg
    s.set_emission(np.zeros((4, 4, 4)))
    assert s.L.names() == ["dcg_set_emission"]


def test_state_buffers_are_checked():
    s = fake_sim()
    refused(s.save_state, np.empty(FakeLib.STATE - 1, np.uint8))
    refused(s.load_state, np.zeros(FakeLib.STATE // 2, np.uint8))
    assert "dcg_save_state" not in s.L.names() and "dcg_load_state" not in s.L.names()
    buf = s.save_state()
    assert buf.size == FakeLib.STATE
    s.load_state(buf)
    assert s.L.names()[-1] == "dcg_load_state"


def test_render_output_is_checked():
    s = fake_sim()
    rp = capi.DcgRenderParams()
    rp.width, rp.height = 8, 6
    refused(s.render, rp, np.empty((8, 6, 3), np.float32))
    img = s.render(rp)
    assert img.shape == (6, 8, 4) and s.L.names() == ["dcg_render"]


def test_topology_arrays_are_checked():
    s = fake_sim(blocks=10)
    ok = dict(pos=np.zeros((10, 4)), parent=np.zeros(10), child=np.zeros((10, 8)), load=[1, 2])
    refused(s.set_topology, dict(ok, pos=np.zeros((9, 4))))
    refused(s.set_topology, dict(ok, child=np.zeros((10, 7))))
    assert not s.L.calls
    s.set_topology(ok)
    assert s.L.names() == ["dcg_set_topology"]


def test_torch_buffers_are_checked():
    torch = pytest.importorskip("torch")
    s = fake_sim()
    n = s.num_cells
    s.get_field("density", torch.empty(n, dtype=torch.float32))  # host tensor: host copy
    assert s.L.calls[-1][1][3] == capi.HOST
    refused(s.get_field, "density", torch.empty(n, dtype=torch.float64))
    refused(s.get_field, "density", torch.empty(2 * n, dtype=torch.float32)[::2])
    # the adjoint works on device memory only
    msg = refused(s.adjoint_step, torch.zeros(n), torch.zeros(n))
    assert "CUDA tensor" in msg
    refused(s.adjoint_dense, np.zeros(16 * 32 * 16, np.float32), np.zeros(n, np.float32))
    assert [c for c in s.L.names() if c.startswith("dcg_adjoint")] == []


def test_batch_emission_is_the_concatenation_of_member_maps():
    from dcgrid_gb300 import sim
    b = object.__new__(sim.Batch)
    b.L, b.h = FakeLib(), C.c_void_p(1)
    b.params = [capi.default_params(16, 16, 16, 50) for _ in range(3)]
    b.params[0].emission_n, b.params[1].emission_n, b.params[2].emission_n = 4, 0, 2
    refused(b.set_emission, np.zeros(64, np.float32))
    b.set_emission(np.zeros(64 + 8, np.float32))
    assert b.L.names() == ["dcg_batch_set_emission"]


def test_reference_render_signature(dcg_lib):
    from dcgrid_gb300 import sim
    for cls in (sim.FluidSimulationDCGrid, sim.FluidSimulationUniform):
        s = fake_sim(cls)
        img = s.render(None, (8, 6), (1.0, 2.0, -3.0), (0.0, 0.6, 0.8), 0.9, (0.0, 1.0, 0.0),
                       channel=capi.RENDER_VELOCITY, shadows=0, smoke_color=(0.1, 0.2, 0.3))
        assert img.shape == (6, 8, 4)
        name, args = s.L.calls[-1]
        assert name == "dcg_render" and args[3] == capi.HOST
        rp = args[1]._obj
        assert (rp.width, rp.height, rp.channel, rp.shadows) == (8, 6, capi.RENDER_VELOCITY, 0)
        assert list(rp.eye) == [1.0, 2.0, -3.0] and list(rp.sun_dir) == [0.0, 1.0, 0.0]
        assert rp.fov == pytest.approx(0.9) and list(rp.smoke_color) == pytest.approx([0.1, 0.2, 0.3])
        assert rp.solids == 1 and rp.aa_samples == 1  # the reference's defaults
        with pytest.raises(TypeError):
            s.render(None, (8, 6), (0, 0, 0), (0, 0, 1), 1.0, (0, 1, 0), colour=1)
        rp2 = capi.DcgRenderParams()
        rp2.width, rp2.height = 4, 4
        assert s.render(rp2).shape == (4, 4, 4)  # the Simulation.render(rp, out) form


def test_reference_named_classes_have_the_reference_methods():
    from dcgrid_gb300 import sim
    # src/fluid_simulation.h:9-22
    methods = ["init", "reset", "adaptTopology", "advectVelocity", "project", "projectLocal", "advectDensity",
               "render", "debugStats"]
    for cls in (sim.FluidSimulationDCGrid, sim.FluidSimulationUniform):
        assert all(callable(getattr(cls, m, None)) for m in methods), cls
