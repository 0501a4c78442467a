"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Only tests, the smoke check and the CPU-baseline leg of bench.py import this
module. It mirrors the product's Python API (dcgrid_gb300.Simulation) so a
parity test can drive both the same way.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from dcgrid_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdcg_oracle.so")
_lib = None


def build(quiet=True):
    """Compiles the oracle with its Makefile (g++, OpenMP)."""
    cmd = ["make", "-s", "-C", HERE]
    subprocess.run(cmd, check=True, capture_output=quiet)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.dcgo_create.argtypes = [C.POINTER(capi.DcgParams), C.c_int32, C.c_int32, C.POINTER(vp)]
        for name in ["dcgo_destroy", "dcgo_reset", "dcgo_advect_velocity", "dcgo_adapt",
                     "dcgo_project", "dcgo_project_local", "dcgo_advect_scalars"]:
            getattr(L, name).argtypes = [vp]
        L.dcgo_step.argtypes = [vp, C.c_int32]
        L.dcgo_add_velocity_noise.argtypes = [vp, C.c_uint64, C.c_float]
        L.dcgo_set_threads.argtypes = [C.c_int32]
        L.dcgo_get_info.argtypes = [vp, C.POINTER(capi.DcgInfo)]
        L.dcgo_last_error_string.argtypes = [vp]
        L.dcgo_last_error_string.restype = C.c_char_p
        L.dcgo_get_field.argtypes = [vp, C.c_int32, vp]
        L.dcgo_set_field.argtypes = [vp, C.c_int32, vp]
        L.dcgo_get_dense.argtypes = [vp, C.c_int32, vp]
        L.dcgo_get_topology.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.dcgo_set_topology.argtypes = [vp, vp, vp, vp, vp, vp]
        L.dcgo_set_apron.argtypes = [vp, vp]
        L.dcgo_get_apron.argtypes = [vp, vp]
        L.dcgo_apron_mismatches.argtypes = [vp]
        L.dcgo_apron_mismatches.restype = C.c_int64
        L.dcgo_get_last_adapt.argtypes = [vp, vp, C.POINTER(C.c_int64), vp, C.POINTER(C.c_int64)]
        L.dcgo_adapt_replay.argtypes = [vp, vp, C.c_int64, vp, C.c_int64]
        L.dcgo_get_scores.argtypes = [vp, vp, vp]
        L.dcgo_get_stats.argtypes = [vp, C.POINTER(capi.DcgStats)]
        L.dcgo_set_emission.argtypes = [vp, vp]
        L.dcgo_set_heightmap.argtypes = [vp, vp, C.c_int32, C.c_int32]
        L.dcgo_render.argtypes = [vp, C.POINTER(capi.DcgRenderParams), vp]
        L.dcgo_adjoint_step.argtypes = [vp, vp, vp, vp]
        L.dcgo_adjoint_dense.argtypes = [vp, vp, vp]
        L.dcgo_adjoint_step_full.argtypes = [vp, vp, vp, vp, vp, C.c_int64, vp, C.c_int64]
        L.dcgo_copy_state.argtypes = [vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class OracleError(RuntimeError):
    pass


class OracleSim:
    """One oracle simulation. precision: 'float' (FP32 mirror) or 'double'."""

    def __init__(self, params, mode=capi.MODE_ADAPTIVE, precision="double"):
        self.L = lib()
        self.params = params
        h = C.c_void_p()
        rc = self.L.dcgo_create(C.byref(params), mode, 0 if precision == "float" else 1, C.byref(h))
        if rc != capi.DCG_OK:
            raise OracleError(f"dcgo_create failed: {capi.STATUS_NAMES.get(rc, rc)}")
        self.h = h
        self.mode = mode
        self.info = capi.DcgInfo()
        self.L.dcgo_get_info(self.h, C.byref(self.info))

    def close(self):
        if self.h:
            self.L.dcgo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != capi.DCG_OK:
            msg = self.L.dcgo_last_error_string(self.h).decode()
            raise OracleError(f"{what}: {capi.STATUS_NAMES.get(rc, rc)} {msg}")

    # stages
    def reset(self): self._chk(self.L.dcgo_reset(self.h), "reset")
    def step(self, n=1): self._chk(self.L.dcgo_step(self.h, n), "step")
    def advect_velocity(self): self._chk(self.L.dcgo_advect_velocity(self.h), "advect_velocity")
    def adapt(self): self._chk(self.L.dcgo_adapt(self.h), "adapt")
    def project(self): self._chk(self.L.dcgo_project(self.h), "project")
    def project_local(self): self._chk(self.L.dcgo_project_local(self.h), "project_local")
    def advect_scalars(self): self._chk(self.L.dcgo_advect_scalars(self.h), "advect_scalars")

    def add_velocity_noise(self, seed, amplitude):
        self._chk(self.L.dcgo_add_velocity_noise(self.h, seed, amplitude), "noise")

    @property
    def num_cells(self):
        return int(self.info.num_cells)

    def set_emission(self, field):
        a = np.ascontiguousarray(field, dtype=np.float64).reshape(-1)
        self._chk(self.L.dcgo_set_emission(self.h, _ptr(a)), "set_emission")

    def set_heightmap(self, heights):
        """(nz, nx) float32 heights (x fastest), or None for the noise terrain;
        resets the simulation."""
        if heights is None:
            self._chk(self.L.dcgo_set_heightmap(self.h, None, 0, 0), "set_heightmap")
            return
        a = np.ascontiguousarray(heights, dtype=np.float32)
        self._chk(self.L.dcgo_set_heightmap(self.h, _ptr(a), a.shape[1], a.shape[0]), "set_heightmap")

    def get_field(self, field):
        fid = capi.FIELD_NAMES[field] if isinstance(field, str) else field
        out = np.empty(self.num_cells, dtype=np.float64)
        self._chk(self.L.dcgo_get_field(self.h, fid, _ptr(out)), "get_field")
        return out

    def set_field(self, field, values):
        fid = capi.FIELD_NAMES[field] if isinstance(field, str) else field
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._chk(self.L.dcgo_set_field(self.h, fid, _ptr(a)), "set_field")

    def get_dense(self, field):
        fid = capi.FIELD_NAMES[field] if isinstance(field, str) else field
        p = self.params
        out = np.empty(p.gx * p.gy * p.gz, dtype=np.float64)
        self._chk(self.L.dcgo_get_dense(self.h, fid, _ptr(out)), "get_dense")
        return out.reshape(p.gz, p.gy, p.gx)

    def get_topology(self):
        B = int(self.info.max_blocks)
        pos = np.empty(4 * B, np.int32)
        parent = np.empty(B, np.uint32)
        child = np.empty(8 * B, np.uint32)
        flags = np.empty(B, np.uint8)
        load = np.zeros(16, np.int64)
        ml = np.zeros(16, np.int64)
        self._chk(self.L.dcgo_get_topology(self.h, _ptr(pos), _ptr(parent), _ptr(child),
                                           _ptr(flags), _ptr(load), _ptr(ml)), "get_topology")
        lv = int(self.info.levels)
        return dict(pos=pos.reshape(B, 4), parent=parent, child=child.reshape(B, 8),
                    flags=flags, load=load[:lv], move_limit=ml[:lv])

    def set_topology(self, topo):
        pos = np.ascontiguousarray(topo["pos"], np.int32)
        parent = np.ascontiguousarray(topo["parent"], np.uint32)
        child = np.ascontiguousarray(topo["child"], np.uint32)
        load = np.zeros(16, np.int64)
        load[: len(topo["load"])] = topo["load"]
        ml = np.zeros(16, np.int64)
        if "move_limit" in topo:
            ml[: len(topo["move_limit"])] = topo["move_limit"]
        self._chk(self.L.dcgo_set_topology(self.h, _ptr(pos), _ptr(parent), _ptr(child),
                                           _ptr(load), _ptr(ml)), "set_topology")

    def get_apron(self):
        B = int(self.info.max_blocks)
        out = np.empty(216 * B, np.int64)
        self._chk(self.L.dcgo_get_apron(self.h, _ptr(out)), "get_apron")
        return out.reshape(B, 216)

    def set_apron(self, apron):
        a = np.ascontiguousarray(apron, np.int64)
        self._chk(self.L.dcgo_set_apron(self.h, _ptr(a)), "set_apron")

    def apron_mismatches(self):
        return int(self.L.dcgo_apron_mismatches(self.h))

    def get_last_adapt(self):
        nm, nr = C.c_int64(), C.c_int64()
        self._chk(self.L.dcgo_get_last_adapt(self.h, None, C.byref(nm), None, C.byref(nr)), "last_adapt")
        moves = np.empty(2 * nm.value, np.int64)
        refines = np.empty(2 * nr.value, np.int64)
        self._chk(self.L.dcgo_get_last_adapt(self.h, _ptr(moves), C.byref(nm), _ptr(refines),
                                             C.byref(nr)), "last_adapt")
        return moves.reshape(-1, 2), refines.reshape(-1, 2)

    def adapt_replay(self, moves, refines):
        m = np.ascontiguousarray(moves, np.int64).reshape(-1)
        r = np.ascontiguousarray(refines, np.int64).reshape(-1)
        self._chk(self.L.dcgo_adapt_replay(self.h, _ptr(m), len(m) // 2, _ptr(r), len(r) // 2),
                  "adapt_replay")

    def get_scores(self):
        B = int(self.info.max_blocks)
        s = np.empty(8 * B, np.float32)
        b = np.empty(B, np.float32)
        self._chk(self.L.dcgo_get_scores(self.h, _ptr(s), _ptr(b)), "scores")
        return s, b

    def stats(self):
        st = capi.DcgStats()
        self._chk(self.L.dcgo_get_stats(self.h, C.byref(st)), "stats")
        return st

    def render(self, rp):
        out = np.empty((rp.height, rp.width, 4), np.float64)
        self._chk(self.L.dcgo_render(self.h, C.byref(rp), _ptr(out)), "render")
        return out

    def adjoint_step(self, lam_in, lam_em=None):
        """FP64 transpose of the step that produced the current state; returns
        the adjoint of the density before it; lam_em is accumulated in place."""
        a = np.ascontiguousarray(lam_in, np.float64)
        out = np.empty_like(a)
        self._chk(self.L.dcgo_adjoint_step(self.h, _ptr(a), _ptr(out), _ptr(lam_em)), "adjoint_step")
        return out

    def adjoint_step_full(self, lam_in, lam_em=None, moves=None, refines=None):
        """FP64 adjoint of one whole step from the state held now (which the
        call advances by the step, replaying `moves` / `refines` when given);
        returns the adjoint of the state before the step ((3 + n_scalars)
        planes) given lam_in, that of the state after it."""
        a = np.ascontiguousarray(lam_in, np.float64)
        out = np.empty_like(a)
        if moves is None:
            mv, nm, rf, nr = None, 0, None, 0
        else:
            mv = np.ascontiguousarray(moves, np.int64).reshape(-1)
            rf = np.ascontiguousarray(refines, np.int64).reshape(-1)
            nm, nr = len(mv) // 2, len(rf) // 2
        self._chk(self.L.dcgo_adjoint_step_full(self.h, _ptr(a), _ptr(out), _ptr(lam_em), _ptr(mv), nm, _ptr(rf),
                                                nr), "adjoint_step_full")
        return out

    def adjoint_dense(self, lam_dense, lam_cells):
        a = np.ascontiguousarray(lam_dense, np.float64).reshape(-1)
        self._chk(self.L.dcgo_adjoint_dense(self.h, _ptr(a), _ptr(lam_cells)), "adjoint_dense")

    def copy_state_from(self, other):
        self._chk(self.L.dcgo_copy_state(self.h, other.h), "copy_state")


def set_threads(n):
    lib().dcgo_set_threads(int(n))
