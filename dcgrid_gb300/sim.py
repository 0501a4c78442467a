"""Python host API over the C ABI (libdcgrid_gb300.so).

Mirrors the reference's simulation interface (src/fluid_simulation.h:4-27):
FluidSimulationDCGrid(size, maxNumBlocks) and FluidSimulationUniform(size)
with init/reset/adaptTopology/advectVelocity/project/projectLocal/
advectDensity/debugStats, plus field and topology accessors the reference
does not expose. Errors raise DcgError carrying the C status code; the
reference would exit(1) instead.
"""
import ctypes as C
import os

import numpy as np

from . import capi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdcgrid_gb300.so")
_lib = None


class DcgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{capi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib():
    """Loads the in-tree CUDA library. There is no fallback: a missing library
    is an error (build it with dcgrid_gb300.build.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing; run dcgrid_gb300.build.build() first")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.dcg_default_params.argtypes = [C.POINTER(capi.DcgParams), C.c_int32, C.c_int32, C.c_int32, C.c_int64]
        L.dcg_default_params.restype = None
        L.dcg_create.argtypes = [C.POINTER(capi.DcgParams), C.c_int32, C.POINTER(vp)]
        for name in ["dcg_destroy", "dcg_reset", "dcg_advect_velocity", "dcg_adapt", "dcg_project",
                     "dcg_project_local", "dcg_advect_scalars", "dcg_sync"]:
            getattr(L, name).argtypes = [vp]
        L.dcg_set_params.argtypes = [vp, C.POINTER(capi.DcgParams)]
        L.dcg_set_mode.argtypes = [C.POINTER(vp), C.c_int32]
        L.dcg_set_stream.argtypes = [vp, vp]
        L.dcg_get_info.argtypes = [vp, C.POINTER(capi.DcgInfo)]
        L.dcg_last_error_string.argtypes = [vp]
        L.dcg_last_error_string.restype = C.c_char_p
        L.dcg_step.argtypes = [vp, C.c_int32]
        L.dcg_add_velocity_noise.argtypes = [vp, C.c_uint64, C.c_float]
        L.dcg_get_field.argtypes = [vp, C.c_int32, vp, C.c_int32]
        L.dcg_set_field.argtypes = [vp, C.c_int32, vp, C.c_int32]
        L.dcg_get_dense.argtypes = [vp, C.c_int32, vp, C.c_int32]
        L.dcg_get_topology.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.dcg_set_topology.argtypes = [vp, vp, vp, vp, vp, vp]
        L.dcg_get_apron.argtypes = [vp, vp]
        L.dcg_get_last_adapt.argtypes = [vp, vp, C.POINTER(C.c_int64), vp, C.POINTER(C.c_int64)]
        L.dcg_get_stats.argtypes = [vp, C.POINTER(capi.DcgStats)]
        L.dcg_set_graphs.argtypes = [vp, C.c_int32]
        L.dcg_time_kernel.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_float),
                                      C.POINTER(C.c_double)]
        L.dcg_launches_per_step.argtypes = [vp, C.POINTER(C.c_int64)]
        L.dcg_set_emission.argtypes = [vp, vp, C.c_int32]
        L.dcg_set_heightmap.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_int32]
        L.dcg_default_render_params.argtypes = [C.POINTER(capi.DcgRenderParams), C.c_int32, C.c_int32]
        L.dcg_default_render_params.restype = None
        L.dcg_render.argtypes = [vp, C.POINTER(capi.DcgRenderParams), vp, C.c_int32]
        L.dcg_state_bytes.argtypes = [vp, C.POINTER(C.c_int64)]
        L.dcg_save_state.argtypes = [vp, vp, C.c_int32]
        L.dcg_load_state.argtypes = [vp, vp, C.c_int32]
        L.dcg_adjoint_step.argtypes = [vp, vp, vp, vp]
        L.dcg_adjoint_dense.argtypes = [vp, vp, vp]
        L.dcg_adjoint_step_full.argtypes = [vp, vp, vp, vp]
        L.dcg_batch_create.argtypes = [C.c_int32, vp, C.POINTER(vp)]
        for name in ["dcg_batch_destroy", "dcg_batch_reset", "dcg_batch_sync"]:
            getattr(L, name).argtypes = [vp]
        L.dcg_batch_step.argtypes = [vp, C.c_int32]
        L.dcg_batch_member.argtypes = [vp, C.c_int32, C.POINTER(vp)]
        L.dcg_batch_set_stream.argtypes = [vp, vp]
        L.dcg_batch_autotune.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(capi.DcgTuning)]
        L.dcg_batch_get_tuning.argtypes = [vp, C.POINTER(capi.DcgTuning)]
        L.dcg_batch_set_tuning.argtypes = [vp, C.POINTER(capi.DcgTuning)]
        L.dcg_batch_get_info.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.dcg_batch_time_solve.argtypes = [vp, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_double)]
        L.dcg_batch_profile_step.argtypes = [vp, vp]
        L.dcg_batch_get_stats.argtypes = [vp, vp]
        L.dcg_batch_set_emission.argtypes = [vp, vp, C.c_int32]
        L.dcg_batch_last_error_string.argtypes = [vp]
        L.dcg_batch_last_error_string.restype = C.c_char_p
        L.dcg_get_dense_noalloc.argtypes = [vp, C.c_int32, vp, C.c_int32]
        L.dcg_plan_bytes.argtypes = [vp, C.c_int32, C.POINTER(C.c_int64)]
        L.dcg_blocks_for_budget.argtypes = [vp, C.c_int64, C.POINTER(C.c_int64)]
        L.dcg_check_div6.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
        L.dcg_check_barrier_timeout.argtypes = [vp, C.c_uint32]
        for name in ["dcg_sizeof_params", "dcg_sizeof_info", "dcg_sizeof_stats", "dcg_sizeof_tuning",
                     "dcg_sizeof_render_params"]:
            getattr(L, name).restype = C.c_size_t
            getattr(L, name).argtypes = []
        _lib = L
    return _lib


def default_params(gx, gy, gz, max_blocks):
    p = capi.DcgParams()
    lib().dcg_default_params(C.byref(p), gx, gy, gz, max_blocks)
    return p


def default_render_params(width, height, params=None):
    """The reference's render defaults; with `params`, the eye is placed in
    front of the domain (-z side) looking along +z at its centre."""
    rp = capi.DcgRenderParams()
    lib().dcg_default_render_params(C.byref(rp), width, height)
    if params is not None:
        dx = params.dx
        rp.eye[0], rp.eye[1], rp.eye[2] = 0.5 * params.gx * dx, 0.5 * params.gy * dx, -1.2 * params.gz * dx
    return rp


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _field_id(field):
    return capi.FIELD_NAMES[field] if isinstance(field, str) else int(field)


def _buf(obj, count, dtype, what, writable=False, device=False):
    """(pointer, capi.HOST | capi.DEVICE) of a C-contiguous numpy array or
    torch tensor of exactly `count` elements of `dtype`. The C library reads or
    writes that many elements behind the pointer, so anything else (wrong size,
    dtype or layout, a read-only output, a host buffer where the call needs
    device memory) raises DcgError(DCG_E_INVALID) before it is called."""
    dt = np.dtype(dtype)
    if hasattr(obj, "data_ptr"):
        got = f"tensor {tuple(obj.shape)} {obj.dtype}{' cuda' if obj.is_cuda else ''}"
        ok = (str(obj.dtype).rsplit(".", 1)[-1] == dt.name and obj.is_contiguous() and obj.numel() == count
              and (obj.is_cuda or not device))
        if ok:
            return C.c_void_p(obj.data_ptr()), (capi.DEVICE if obj.is_cuda else capi.HOST)
    elif isinstance(obj, np.ndarray):
        got = f"array {obj.shape} {obj.dtype}"
        ok = (obj.dtype == dt and obj.flags.c_contiguous and obj.size == count and not device
              and (obj.flags.writeable or not writable))
        if ok:
            return _ptr(obj), capi.HOST
    else:
        got = type(obj).__name__
    where = "CUDA tensor" if device else "array or tensor"
    raise DcgError(capi.DCG_E_INVALID, f"{what}: expected a contiguous {dt.name} {where} of {count} elements, got {got}")


class Simulation:
    """One simulation handle (adaptive or uniform)."""

    def __init__(self, params, mode=capi.MODE_ADAPTIVE):
        self.L = lib()
        self.params = params
        h = C.c_void_p()
        rc = self.L.dcg_create(C.byref(params), mode, C.byref(h))
        if rc != capi.DCG_OK:
            raise DcgError(rc, "dcg_create failed")
        self.h = h
        self.mode = mode
        self.info = capi.DcgInfo()
        self._chk(self.L.dcg_get_info(self.h, C.byref(self.info)), "get_info")

    # -- lifecycle --------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.L.dcg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, rc, what):
        if rc != capi.DCG_OK:
            msg = self.L.dcg_last_error_string(self.h).decode() if self.h else ""
            raise DcgError(rc, f"{what}: {msg}")

    def reset(self):
        self._chk(self.L.dcg_reset(self.h), "reset")

    def set_params(self, params):
        self._chk(self.L.dcg_set_params(self.h, C.byref(params)), "set_params")
        self.params = params

    def set_mode(self, mode):
        """The reference's adaptive/uniform switch: recreate, state dropped."""
        self._chk(self.L.dcg_set_mode(C.byref(self.h), mode), "set_mode")
        self.mode = mode
        self._chk(self.L.dcg_get_info(self.h, C.byref(self.info)), "get_info")

    def set_stream(self, stream_ptr):
        self._chk(self.L.dcg_set_stream(self.h, C.c_void_p(stream_ptr)), "set_stream")

    def set_graphs(self, on):
        self._chk(self.L.dcg_set_graphs(self.h, 1 if on else 0), "set_graphs")

    # -- the step and its stages ------------------------------------------
    def step(self, n=1):
        self._chk(self.L.dcg_step(self.h, n), "step")

    def advect_velocity(self):
        self._chk(self.L.dcg_advect_velocity(self.h), "advect_velocity")

    def adapt(self):
        self._chk(self.L.dcg_adapt(self.h), "adapt")

    def project(self):
        self._chk(self.L.dcg_project(self.h), "project")

    def project_local(self):
        self._chk(self.L.dcg_project_local(self.h), "project_local")

    def advect_scalars(self):
        self._chk(self.L.dcg_advect_scalars(self.h), "advect_scalars")

    def sync(self):
        self._chk(self.L.dcg_sync(self.h), "sync")

    def set_emission(self, field):
        """Emission field (emission_n^3, x fastest) from a host array or a CUDA
        torch tensor (pinned host tensors are copied asynchronously)."""
        n = int(self.params.emission_n) ** 3
        a = field if hasattr(field, "data_ptr") else np.ascontiguousarray(field, np.float32)
        if n == 0:  # no emission map: the library reports it
            self._chk(self.L.dcg_set_emission(self.h, _ptr(np.zeros(1, np.float32)), capi.HOST), "set_emission")
        ptr, where = _buf(a, n, np.float32, "set_emission")
        if where == capi.HOST:
            self._emis_keep = a  # an asynchronous copy may still read it
        self._chk(self.L.dcg_set_emission(self.h, ptr, where), "set_emission")

    def set_heightmap(self, heights):
        """Terrain from a (nz, nx) heightmap (x fastest; a host array or CUDA
        torch tensor) instead of the value noise: height = terrain_base_height
        + terrain_amplitude * bilinear sample. None restores the noise terrain.
        Resets the simulation."""
        if heights is None:
            self._chk(self.L.dcg_set_heightmap(self.h, None, 0, 0, capi.HOST), "set_heightmap")
            return
        a = heights if hasattr(heights, "data_ptr") else np.ascontiguousarray(heights, np.float32)
        if len(a.shape) != 2:
            raise DcgError(capi.DCG_E_INVALID, f"set_heightmap: expected (nz, nx) heights, got shape {tuple(a.shape)}")
        nz, nx = int(a.shape[0]), int(a.shape[1])
        ptr, where = _buf(a, nx * nz, np.float32, "set_heightmap")
        self._chk(self.L.dcg_set_heightmap(self.h, ptr, nx, nz, where), "set_heightmap")

    def add_velocity_noise(self, seed, amplitude):
        self._chk(self.L.dcg_add_velocity_noise(self.h, seed, amplitude), "noise")

    # -- access -----------------------------------------------------------
    @property
    def num_cells(self):
        return int(self.info.num_cells)

    def get_field(self, field, out=None):
        """Host copy (float32 numpy) in the canonical layout, or, when `out` is a
        CUDA torch tensor, a device-to-device copy into it."""
        fid = _field_id(field)
        a = np.empty(self.num_cells, np.float32) if out is None else out
        ptr, where = _buf(a, self.num_cells, np.float32, "get_field", writable=True)
        self._chk(self.L.dcg_get_field(self.h, fid, ptr, where), "get_field")
        return a

    def set_field(self, field, values):
        fid = _field_id(field)
        a = values if hasattr(values, "data_ptr") else np.ascontiguousarray(values, np.float32)
        ptr, where = _buf(a, self.num_cells, np.float32, "set_field")
        self._chk(self.L.dcg_set_field(self.h, fid, ptr, where), "set_field")

    def get_dense(self, field):
        p = self.params
        a = np.empty(p.gx * p.gy * p.gz, np.float32)
        self._chk(self.L.dcg_get_dense(self.h, _field_id(field), _ptr(a), capi.HOST), "get_dense")
        return a.reshape(p.gz, p.gy, p.gx)

    def get_dense_noalloc(self, field, out=None):
        """get_dense without a device allocation (dcg_get_dense_noalloc): for
        hosts that cap the library's device memory up front. Domains above 2^20
        finest cells are refused. `out`: a host array or CUDA tensor of
        gx*gy*gz float32 (returned as given), else a new (gz, gy, gx) array."""
        p = self.params
        n = p.gx * p.gy * p.gz
        a = np.empty(n, np.float32) if out is None else out
        ptr, where = _buf(a, n, np.float32, "get_dense_noalloc", writable=True)
        self._chk(self.L.dcg_get_dense_noalloc(self.h, _field_id(field), ptr, where), "get_dense_noalloc")
        return a.reshape(p.gz, p.gy, p.gx) if out is None else a

    def get_topology(self):
        B = int(self.info.max_blocks)
        lv = int(self.info.levels)
        pos = np.empty(4 * B, np.int32)
        parent = np.empty(B, np.uint32)
        child = np.empty(8 * B, np.uint32)
        flags = np.empty(B, np.uint8)
        load = np.zeros(16, np.int64)
        ml = np.zeros(16, np.int64)
        self._chk(self.L.dcg_get_topology(self.h, _ptr(pos), _ptr(parent), _ptr(child), _ptr(flags),
                                          _ptr(load), _ptr(ml)), "get_topology")
        return dict(pos=pos.reshape(B, 4), parent=parent, child=child.reshape(B, 8), flags=flags,
                    load=load[:lv], move_limit=ml[:lv])

    def set_topology(self, topo):
        B = int(self.info.max_blocks)
        pos = np.ascontiguousarray(topo["pos"], np.int32)
        parent = np.ascontiguousarray(topo["parent"], np.uint32)
        child = np.ascontiguousarray(topo["child"], np.uint32)
        _buf(pos, 4 * B, np.int32, "set_topology pos")
        _buf(parent, B, np.uint32, "set_topology parent")
        _buf(child, 8 * B, np.uint32, "set_topology child")
        load = np.zeros(16, np.int64)
        load[: len(topo["load"])] = topo["load"]
        ml = np.zeros(16, np.int64)
        if "move_limit" in topo:
            ml[: len(topo["move_limit"])] = topo["move_limit"]
        self._chk(self.L.dcg_set_topology(self.h, _ptr(pos), _ptr(parent), _ptr(child), _ptr(load), _ptr(ml)),
                  "set_topology")

    def get_apron(self):
        B = int(self.info.max_blocks)
        a = np.empty(216 * B, np.int64)
        self._chk(self.L.dcg_get_apron(self.h, _ptr(a)), "get_apron")
        return a.reshape(B, 216)

    def get_last_adapt(self):
        nm, nr = C.c_int64(), C.c_int64()
        self._chk(self.L.dcg_get_last_adapt(self.h, None, C.byref(nm), None, C.byref(nr)), "last_adapt")
        moves = np.empty(2 * nm.value, np.int64)
        refines = np.empty(2 * nr.value, np.int64)
        self._chk(self.L.dcg_get_last_adapt(self.h, _ptr(moves), C.byref(nm), _ptr(refines), C.byref(nr)),
                  "last_adapt")
        return moves.reshape(-1, 2), refines.reshape(-1, 2)

    def time_kernel(self, which, level=0, reps=20):
        """(mean ms per launch, algorithmic bytes per launch) of one kernel."""
        ms, by = C.c_float(), C.c_double()
        self._chk(self.L.dcg_time_kernel(self.h, which, level, reps, C.byref(ms), C.byref(by)), "time_kernel")
        return float(ms.value), float(by.value)

    def launches_per_step(self):
        n = C.c_int64()
        self._chk(self.L.dcg_launches_per_step(self.h, C.byref(n)), "launches_per_step")
        return int(n.value)

    # -- headless renderer ---------------------------------------------------
    def render(self, rp, out=None):
        """RGBA image (height, width, 4) float32: numpy (host) or a CUDA torch
        tensor given as `out`."""
        if out is None:
            out = np.empty((max(rp.height, 0), max(rp.width, 0), 4), np.float32)
        ptr, where = _buf(out, max(rp.height, 0) * max(rp.width, 0) * 4, np.float32, "render", writable=True)
        self._chk(self.L.dcg_render(self.h, C.byref(rp), ptr, where), "render")
        return out

    # -- state I/O (checkpoint / resume) ------------------------------------
    def state_bytes(self):
        n = C.c_int64()
        self._chk(self.L.dcg_state_bytes(self.h, C.byref(n)), "state_bytes")
        return n.value

    def save_state(self, out=None):
        """The state a step depends on, into a uint8 buffer: a numpy array (host)
        or a CUDA torch tensor (device); a new host array when out is None."""
        n = self.state_bytes()
        if out is None:
            out = np.empty(n, np.uint8)
        ptr, where = _buf(out, n, np.uint8, "save_state", writable=True)
        self._chk(self.L.dcg_save_state(self.h, ptr, where), "save_state")
        return out

    def load_state(self, buf):
        a = buf if hasattr(buf, "data_ptr") else np.ascontiguousarray(buf, np.uint8)
        ptr, where = _buf(a, self.state_bytes(), np.uint8, "load_state")
        self._chk(self.L.dcg_load_state(self.h, ptr, where), "load_state")

    def save(self, path):
        """Writes the state to a file (checkpoint)."""
        self.save_state().tofile(path)

    def load(self, path):
        self.load_state(np.fromfile(path, np.uint8))

    # -- adjoint of the density path (CUDA torch tensors) --------------------
    def adjoint_step(self, lam_in, lam_out, lam_emission=None):
        """lam_out <- transpose of the last step's density map applied to
        lam_in; lam_emission (emission_n^3) accumulates the emission adjoint."""
        n = self.num_cells
        li, _ = _buf(lam_in, n, np.float32, "adjoint_step lam_in", device=True)
        lo, _ = _buf(lam_out, n, np.float32, "adjoint_step lam_out", device=True)
        em = None
        if lam_emission is not None and self.params.emission_n > 0:
            em, _ = _buf(lam_emission, int(self.params.emission_n) ** 3, np.float32, "adjoint_step lam_emission",
                         device=True)
        self._chk(self.L.dcg_adjoint_step(self.h, li, lo, em), "adjoint_step")

    def adjoint_step_full(self, lam_in, lam_out, lam_emission=None):
        """dcg_adjoint_step_full: the handle holds the state before a step; the
        call runs the step and writes into lam_out the adjoint of that state
        (velocity and scalars, (3 + n_scalars) planes of num_cells) given
        lam_in, the adjoint of the state after it; lam_emission accumulates
        the emission map's adjoint."""
        n = (3 + int(self.params.n_scalars)) * self.num_cells
        li, _ = _buf(lam_in, n, np.float32, "adjoint_step_full lam_in", device=True)
        lo, _ = _buf(lam_out, n, np.float32, "adjoint_step_full lam_out", device=True)
        em = None
        if lam_emission is not None and self.params.emission_n > 0:
            em, _ = _buf(lam_emission, int(self.params.emission_n) ** 3, np.float32,
                         "adjoint_step_full lam_emission", device=True)
        self._chk(self.L.dcg_adjoint_step_full(self.h, li, lo, em), "adjoint_step_full")

    def adjoint_dense(self, lam_dense, lam_cells):
        p = self.params
        ld, _ = _buf(lam_dense, p.gx * p.gy * p.gz, np.float32, "adjoint_dense lam_dense", device=True)
        lc, _ = _buf(lam_cells, self.num_cells, np.float32, "adjoint_dense lam_cells", device=True)
        self._chk(self.L.dcg_adjoint_dense(self.h, ld, lc), "adjoint_dense")

    def stats(self):
        st = capi.DcgStats()
        self._chk(self.L.dcg_get_stats(self.h, C.byref(st)), "stats")
        return st


def _reference_render(sim, dest, resolution, eyePos, eyeDir, fov, sunDir, switches):
    """FluidSimulation::render(dest, resolution, eyePos, eyeDir, fov, sunDir)
    (src/fluid_simulation.h:18-20). The reference writes float4 texels into a
    CUDA surface (dcgrid/dcgrid_rendering.cu:91); here `dest` is a (height,
    width, 4) float32 numpy array or CUDA tensor, or None for a new host image.
    The reference reads its render switches from SimParams; `switches` sets
    the matching dcg_render_params fields (channel, shadows, solids, precise,
    aa_samples, ambient, smoke_color, scene_color, floor_color), the rest keep
    the reference's defaults."""
    width, height = int(resolution[0]), int(resolution[1])
    rp = default_render_params(width, height)
    for name, v in (("eye", eyePos), ("eye_dir", eyeDir), ("sun_dir", sunDir)):
        arr = getattr(rp, name)
        for i in range(3):
            arr[i] = float(v[i])
    rp.fov = float(fov)
    for name, v in switches.items():
        if name not in ("channel", "shadows", "solids", "precise", "aa_samples", "ambient", "smoke_color",
                        "scene_color", "floor_color"):
            raise TypeError(f"render: unknown switch {name!r}")
        if name.endswith("_color"):
            arr = getattr(rp, name)
            for i in range(3):
                arr[i] = float(v[i])
        else:
            setattr(rp, name, v)
    return Simulation.render(sim, rp, dest)


class FluidSimulationDCGrid(Simulation):
    """FluidSimulationDCGrid(const int3 &size, const size_t &maxNumBlocks)
    (src/dcgrid/fluid_simulation_dcgrid.h:7) with the reference's method names."""

    def __init__(self, size, maxNumBlocks, params=None):
        p = params if params is not None else default_params(size[0], size[1], size[2], maxNumBlocks)
        p.gx, p.gy, p.gz = size
        p.max_blocks = maxNumBlocks
        super().__init__(p, capi.MODE_ADAPTIVE)

    def init(self):
        self.reset()

    def adaptTopology(self):
        self.adapt()

    def advectVelocity(self):
        self.advect_velocity()

    def projectLocal(self):
        self.project_local()

    def advectDensity(self):
        self.advect_scalars()

    def render(self, dest, resolution=None, eyePos=None, eyeDir=None, fov=None, sunDir=None, **switches):
        """The reference's render(dest, resolution, eyePos, eyeDir, fov,
        sunDir) (fluid_simulation_dcgrid.cu:485); given a DcgRenderParams
        first, Simulation.render(rp, out)."""
        if isinstance(dest, capi.DcgRenderParams):
            return Simulation.render(self, dest, resolution)
        return _reference_render(self, dest, resolution, eyePos, eyeDir, fov, sunDir, switches)

    def debugStats(self):
        return self.stats().residual


class FluidSimulationUniform(Simulation):
    """FluidSimulationUniform(const int3 &size) (fluid_simulation_uniform.h:7)."""

    def __init__(self, size, params=None):
        p = params if params is not None else default_params(size[0], size[1], size[2], 0)
        p.gx, p.gy, p.gz = size
        super().__init__(p, capi.MODE_UNIFORM)

    def init(self):
        self.reset()

    def adaptTopology(self):
        self.adapt()

    def advectVelocity(self):
        self.advect_velocity()

    def projectLocal(self):
        self.project_local()

    def advectDensity(self):
        self.advect_scalars()

    def render(self, dest, resolution=None, eyePos=None, eyeDir=None, fov=None, sunDir=None, **switches):
        """The reference's render(dest, resolution, eyePos, eyeDir, fov,
        sunDir) (fluid_simulation_uniform.cu:149); given a DcgRenderParams
        first, Simulation.render(rp, out)."""
        if isinstance(dest, capi.DcgRenderParams):
            return Simulation.render(self, dest, resolution)
        return _reference_render(self, dest, resolution, eyePos, eyeDir, fov, sunDir, switches)

    def debugStats(self):
        return self.stats().mass


class _Member(Simulation):
    """Borrowed handle of one batch member: field, stats, topology and
    emission access; the batch steps and owns it."""

    def __init__(self, batch, handle, params):
        self.L = lib()
        self.params = params
        self.h = handle
        self.mode = capi.MODE_ADAPTIVE
        self._batch = batch  # keeps the owner alive
        self.info = capi.DcgInfo()
        self._chk(self.L.dcg_get_info(self.h, C.byref(self.info)), "get_info")

    def close(self):
        self.h = None


class Batch:
    """Many independent adaptive simulations stepped together (dcg_batch_*):
    one launch per field stage over all members, one cooperative launch per
    cascade round, member adaptations as parallel graph branches."""

    def __init__(self, params_list):
        self.L = lib()
        self.params = list(params_list)
        arr = (capi.DcgParams * len(self.params))(*self.params)
        h = C.c_void_p()
        rc = self.L.dcg_batch_create(len(self.params), C.cast(arr, C.c_void_p), C.byref(h))
        if rc != capi.DCG_OK:
            raise DcgError(rc, "dcg_batch_create failed")
        self.h = h
        self.members = []
        for i, p in enumerate(self.params):
            mh = C.c_void_p()
            self._chk(self.L.dcg_batch_member(self.h, i, C.byref(mh)), "member")
            self.members.append(_Member(self, mh, p))

    def _chk(self, rc, what):
        if rc != capi.DCG_OK:
            msg = self.L.dcg_batch_last_error_string(self.h).decode() if self.h else ""
            raise DcgError(rc, f"{what}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.close()
            self.L.dcg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.members)

    def __getitem__(self, i):
        return self.members[i]

    def reset(self):
        self._chk(self.L.dcg_batch_reset(self.h), "reset")

    def step(self, n=1):
        self._chk(self.L.dcg_batch_step(self.h, n), "step")

    def sync(self):
        self._chk(self.L.dcg_batch_sync(self.h), "sync")

    def set_stream(self, stream_ptr):
        self._chk(self.L.dcg_batch_set_stream(self.h, C.c_void_p(stream_ptr)), "set_stream")

    def autotune(self, spinup_steps=10, reps=3):
        t = capi.DcgTuning()
        self._chk(self.L.dcg_batch_autotune(self.h, spinup_steps, reps, C.byref(t)), "autotune")
        return capi.tuning_to_dict(t)

    def get_tuning(self):
        t = capi.DcgTuning()
        self._chk(self.L.dcg_batch_get_tuning(self.h, C.byref(t)), "get_tuning")
        return t

    def set_tuning(self, t):
        self._chk(self.L.dcg_batch_set_tuning(self.h, C.byref(t)), "set_tuning")

    def info(self):
        n, nb, nl = C.c_int32(), C.c_int64(), C.c_int64()
        self._chk(self.L.dcg_batch_get_info(self.h, C.byref(n), C.byref(nb), C.byref(nl)), "get_info")
        return {"n": n.value, "device_bytes": nb.value, "launches_per_step": nl.value}

    def set_emission(self, maps):
        """Every member's emission map in one copy: the maps of the members with
        emission_n > 0, in member order, as one contiguous host array or CUDA
        torch tensor (pinned host tensors are copied asynchronously)."""
        n = sum(int(p.emission_n) ** 3 for p in self.params)
        a = maps if hasattr(maps, "data_ptr") else np.ascontiguousarray(maps, np.float32)
        if n == 0:  # no member has an emission map: the library reports it
            self._chk(self.L.dcg_batch_set_emission(self.h, _ptr(np.zeros(1, np.float32)), capi.HOST),
                      "set_emission")
        ptr, where = _buf(a, n, np.float32, "set_emission")
        if where == capi.HOST:
            self._emis_keep = a  # an asynchronous copy may still read it
        self._chk(self.L.dcg_batch_set_emission(self.h, ptr, where), "set_emission")

    def stats(self):
        """dcg_get_stats of every member, with one synchronisation."""
        arr = (capi.DcgStats * len(self.members))()
        self._chk(self.L.dcg_batch_get_stats(self.h, C.cast(arr, C.c_void_p)), "stats")
        return list(arr)

    STAGES = ("advect_velocity", "adapt", "divergence", "cascade", "apply_pressure", "advect_scalars", "step")

    def profile_step(self):
        """One step outside the step graph, timed per stage (dcg_batch_profile_step):
        a dict of milliseconds per stage and for the whole step."""
        ms = (C.c_float * 7)()
        self._chk(self.L.dcg_batch_profile_step(self.h, C.cast(ms, C.c_void_p)), "profile_step")
        return dict(zip(self.STAGES, [float(x) for x in ms]))

    def time_solve(self, reps=5):
        ms, b = C.c_float(), C.c_double()
        self._chk(self.L.dcg_batch_time_solve(self.h, reps, C.byref(ms), C.byref(b)), "time_solve")
        return ms.value, b.value
