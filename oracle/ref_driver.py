"""Runs the reference's own CUDA kernels headless on a GPU (TEST INFRASTRUCTURE).

The kernels come from oracle/_ref/ref_dcgrid.cubin (built from the reference
sources by oracle/build_ref.sh) and are launched through the CUDA driver API.
This file restates only the reference's host orchestration of
src/dcgrid/fluid_simulation_dcgrid.cu (allocation, reset/init, stage launch
sequences, the host-side candidate ranking of moveBlocks/refineSubblocks) so
the kernels run as they do inside the reference application. Equal keys in the
host ranking are ordered by index, as the oracle does.

Used only to generate the golden fixtures under tests/golden/.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
FLT_MAX = np.float32(3.4028234663852886e38)
SIZE_MAX = np.uint64(0xFFFFFFFFFFFFFFFF)


class SimParams(C.Structure):
    """src/data/sim_params.h:14-47"""
    _fields_ = [("dt", C.c_float), ("gx", C.c_int), ("gy", C.c_int), ("gz", C.c_int),
                ("dx", C.c_float), ("rdx", C.c_float),
                ("velocity_emission_rate", C.c_float), ("density_emission_rate", C.c_float),
                ("emission_radius", C.c_float),
                ("enable_additional_solids", C.c_bool), ("render_solids", C.c_bool),
                ("render_shadows", C.c_bool), ("render_precise", C.c_bool),
                ("render_channel", C.c_int), ("aa_samples", C.c_float), ("ambient", C.c_float),
                ("background_color", C.c_float * 3), ("floor_color", C.c_float * 3),
                ("smoke_color", C.c_float * 3), ("scene_color", C.c_float * 3)]


class DCGridStruct(C.Structure):
    """struct DCGrid (src/dcgrid/dcgrid.h:5-43)"""
    _fields_ = [("maxNumBlocks", C.c_uint64), ("levels", C.c_int), ("sparseLevels", C.c_int)] + \
               [(n, C.c_uint64) for n in [
                   "maxNumBlocksLevel", "fullBlocksLevel", "blockLoads", "levelOffsets", "hashTableSize",
                   "hashTableOffset", "hashKey", "hashVal", "blockPositions", "blockLevels", "cellIndices",
                   "freeBlockIndices", "blockFlags", "parentIndices", "childIndices", "density", "velocity",
                   "fluidity", "temporary", "t_velocity", "vorticity", "divergence", "pressure", "t_pressure",
                   "t_density"]]


def sim_params_from(p):
    """SimParams with the physics of a dcg_params (reference defaults otherwise)."""
    sp = SimParams()
    sp.dt, sp.gx, sp.gy, sp.gz, sp.dx = p.dt, p.gx, p.gy, p.gz, p.dx
    sp.rdx = np.float32(1.0) / np.float32(p.dx)
    sp.velocity_emission_rate = p.velocity_emission_rate
    sp.density_emission_rate = p.density_emission_rate
    sp.emission_radius = p.emission_radius if p.inlet_enabled else -1.0
    sp.enable_additional_solids = bool(p.solids & 1)
    sp.aa_samples = 1.0
    return sp


class Driver:
    """Minimal CUDA driver API over ctypes, sharing torch's primary context."""

    def __init__(self, cubin):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")
        self.torch = torch
        self.cu = C.CDLL("libcuda.so.1")
        self._chk(self.cu.cuInit(0), "cuInit")
        ctx = C.c_void_p()
        self._chk(self.cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            dev = C.c_int()
            self._chk(self.cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
            self._chk(self.cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev), "retain")
            self._chk(self.cu.cuCtxSetCurrent(ctx), "set current")
        data = open(cubin, "rb").read()
        self._img = C.create_string_buffer(data, len(data))
        self.mod = C.c_void_p()
        self._chk(self.cu.cuModuleLoadData(C.byref(self.mod), self._img), "cuModuleLoadData")
        names = open(os.path.join(REF_DIR, "ref_names.txt")).read().split()
        self.fn = {}
        for n in names:
            f = C.c_void_p()
            if self.cu.cuModuleGetFunction(C.byref(f), self.mod, n.encode()) == 0:
                # Itanium mangling: _Z<len><identifier><parameter types>
                i = 2
                while n[i].isdigit():
                    i += 1
                self.fn[n[i:i + int(n[2:i])]] = f

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUresult {rc}")

    def global_ptr(self, name):
        p, sz = C.c_uint64(), C.c_size_t()
        self._chk(self.cu.cuModuleGetGlobal_v2(C.byref(p), C.byref(sz), self.mod, name.encode()), "global")
        return p.value, sz.value

    def launch(self, name, grid, block, *args):
        f = self.fn[name]
        grid = grid if isinstance(grid, tuple) else (grid, 1, 1)
        block = block if isinstance(block, tuple) else (block, 1, 1)
        if min(grid) <= 0:
            return
        holders = [a if isinstance(a, C._SimpleCData) else C.c_uint64(a) for a in args]
        params = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
        self._chk(self.cu.cuLaunchKernel(f, grid[0], grid[1], grid[2], block[0], block[1], block[2], 0,
                                         None, params, None), f"launch {name}")

    def sync(self):
        self._chk(self.cu.cuCtxSynchronize(), "sync")


def idiv_up(a, b):
    return a // b + (1 if a % b else 0)


class RefDCGrid:
    """FluidSimulationDCGrid (fluid_simulation_dcgrid.cu:9-529) over the
    reference's kernels. `levels` overrides the derived level count."""

    def __init__(self, drv, params, levels=None, init_passes=5):
        import torch
        self.init_passes = init_passes
        self.d, self.t = drv, torch
        self.p = params
        size = (params.gx, params.gy, params.gz)
        maxNumBlocks = int(params.max_blocks)
        minDim = min(size)
        cellSize, lv = 2, 1
        while all(s % cellSize == 0 for s in size) and cellSize * 4 <= minDim:
            lv += 1
            cellSize *= 2
        lv = levels or (params.levels if params.levels > 0 else lv)
        self.levels = lv
        self.full = [idiv_up(size[0], cs * 4) * idiv_up(size[1], cs * 4) * idiv_up(size[2], cs * 4)
                     for cs in [1 << l for l in range(lv)]]
        if maxNumBlocks < self.full[-1]:
            raise ValueError("too few blocks")
        self.maxL = [0] * lv
        self.maxL[-1] = self.full[-1]
        left = maxNumBlocks - self.maxL[-1]
        for l in range(lv - 2, -1, -1):
            self.maxL[l] = min(left // (l + 1), self.full[l])
            left -= self.maxL[l]
        self.off = [0] * lv
        for l in range(1, lv):
            self.off[l] = self.off[l - 1] + self.maxL[l - 1]
        self.sparse = 0
        for l in range(lv):
            if self.maxL[l] < self.full[l]:
                self.sparse = l + 1
        self.B = maxNumBlocks
        self.gridSize = idiv_up(maxNumBlocks, 256)
        self.hashTableSize = 4 * maxNumBlocks
        self.numCells = 64 * maxNumBlocks
        B, N = self.B, self.numCells
        dev = "cuda"
        u8 = lambda n: torch.zeros(max(int(n), 16), dtype=torch.uint8, device=dev)
        self.buf = dict(
            density=u8(N * 4), velocity=u8(N * 12), fluidity=u8(N * 4), temporary=u8(N * 12),
            hashTableSize=u8(lv * 8), hashTableOffset=u8(lv * 8), hashKey=u8(self.hashTableSize * 4),
            hashVal=u8(self.hashTableSize * 8), blockPositions=u8(B * 12), blockLevels=u8(B),
            blockFlags=u8(B), parentIndices=u8(B * 8), cellIndices=u8(B * 216 * 8), childIndices=u8(8 * B * 8),
            maxNumBlocksLevel=u8(lv * 8), fullBlocksLevel=u8(lv * 8), levelOffsets=u8(lv * 8),
            freeBlockIndices=u8(B * 8), blockLoads=u8(lv * 8),
            subScores=u8(8 * B * 4), blockScores=u8(B * 4), blockIdx=u8(B * 8), destIdx=u8(8 * B * 8),
            touched=u8(B * 8 * 2))
        self.h = DCGridStruct()
        self.h.maxNumBlocks, self.h.levels, self.h.sparseLevels = B, lv, self.sparse
        for name, _ in DCGridStruct._fields_[3:]:
            if name in self.buf:
                setattr(self.h, name, self.buf[name].data_ptr())
        self.d_grid = u8(C.sizeof(DCGridStruct))
        self._h2d("hashTableSize", np.array([4 * m for m in self.maxL], np.uint64))
        hoff = np.zeros(lv, np.uint64)
        for l in range(1, lv):
            hoff[l] = hoff[l - 1] + 4 * self.maxL[l - 1]
        self._h2d("hashTableOffset", hoff)
        self._h2d("maxNumBlocksLevel", np.array(self.maxL, np.uint64))
        self._h2d("fullBlocksLevel", np.array(self.full, np.uint64))
        self._h2d("levelOffsets", np.array(self.off, np.uint64))
        sp = sim_params_from(params)
        ptr, sz = drv.global_ptr("params")
        assert sz == C.sizeof(SimParams), (sz, C.sizeof(SimParams))
        drv._chk(drv.cu.cuMemcpyHtoD_v2(C.c_uint64(ptr), C.byref(sp), C.c_size_t(sz)), "params")
        self.moveLimit = [0] * lv
        self.reset()

    # -- memory helpers
    def _h2d(self, name, arr):
        a = np.ascontiguousarray(arr)
        t = self.buf[name]
        t[: a.nbytes].copy_(self.t.from_numpy(a.view(np.uint8).reshape(-1)))

    def _d2h(self, name, dtype, count):
        n = np.dtype(dtype).itemsize * count
        return self.buf[name][:n].cpu().numpy().view(dtype).copy()

    def _memset(self, name, val, nbytes=None):
        t = self.buf[name]
        (t if nbytes is None else t[:nbytes]).fill_(val)

    @property
    def g(self):
        return self.d_grid.data_ptr()

    # -- FluidSimulationDCGrid::reset / init (cu:190-261)
    def reset(self):
        B, lv = self.B, self.levels
        self._memset("hashKey", 0xFF)
        self._memset("hashVal", 0xFF)
        self._memset("blockPositions", 0)
        self._memset("blockLevels", 0xFF)
        self._memset("blockFlags", 0)
        self._memset("parentIndices", 0xFF)
        self._memset("childIndices", 0xFF)
        self._memset("cellIndices", 0)
        for n in ["density", "velocity", "fluidity", "temporary"]:
            self._memset(n, 0)
        loads = [self.maxL[l] if self.maxL[l] == self.full[l] else 0 for l in range(lv)]
        self.moveLimit = [0] * lv
        self._h2d("blockLoads", np.array(loads, np.uint64))
        self._h2d("freeBlockIndices", np.arange(B, dtype=np.uint64))
        raw = bytes(self.h)
        self.d_grid[: len(raw)].copy_(self.t.frombuffer(bytearray(raw), dtype=self.t.uint8))
        self.d.launch("k_dcgrid_init_aliasses", 1, 1, self.g)
        self.d.sync()
        self.init()

    def init(self):
        self.d.launch("k_dcgrid_init_apron_indices", self.gridSize, 256, self.g)
        for level in range(self.sparse, self.levels):
            ext = 4 << level
            rx, ry, rz = (idiv_up(self.p.gx, ext), idiv_up(self.p.gy, ext), idiv_up(self.p.gz, ext))
            self.d.launch("k_dcgrid_activate_level", (idiv_up(rx, 4), idiv_up(ry, 4), idiv_up(rz, 4)), (4, 4, 4),
                          self.g, C.c_uint8(level))
        self.d.sync()
        for _ in range(self.init_passes):  # the reference runs 5 (cu:207-209)
            self.adaptTopology()

    # -- stages (cu:263-318)
    def _accumulate(self, kernel):
        for level in range(self.levels - 1):
            self.d.launch(kernel, idiv_up(self.maxL[level] * 8, 64), 64, self.g, C.c_uint8(level))

    def advectVelocity(self):
        self.d.launch("k_dcgrid_advect_velocity", self.B, 64, self.g)
        self.buf["velocity"].copy_(self.buf["temporary"])
        self._accumulate("k_dcgrid_accumulate_velocity")
        self.d.sync()

    def project(self):
        # the reference hard-wires 5 pairs of sweeps per level (cu:274-290);
        # other sweep counts come from params.jacobi_iters (10 = the reference)
        pairs = max(self.p.jacobi_iters, 0) // 2
        self.d.launch("k_dcgrid_calc_divergence", self.B, 64, self.g)
        self._accumulate("k_dcgrid_accumulate_divergence")
        top = self.levels - 1
        for _ in range(pairs):
            self.d.launch("k_dcgrid_jacobi", self.maxL[top], 64, self.g, C.c_uint8(top))
            self.d.launch("k_dcgrid_jacobi_inv", self.maxL[top], 64, self.g, C.c_uint8(top))
        for level in range(self.levels - 2, -1, -1):
            self.d.launch("k_dcgrid_prolongate", self.maxL[level], 64, self.g, C.c_uint8(level))
            for _ in range(pairs):
                self.d.launch("k_dcgrid_jacobi", self.maxL[level], 64, self.g, C.c_uint8(level))
                self.d.launch("k_dcgrid_jacobi_inv", self.maxL[level], 64, self.g, C.c_uint8(level))
        self.d.launch("k_dcgrid_apply_pressure", self.B, 64, self.g)
        self._accumulate("k_dcgrid_accumulate_velocity")
        self.d.sync()

    def projectLocal(self):
        self.d.launch("k_dcgrid_calc_divergence", self.B, 64, self.g)
        self._accumulate("k_dcgrid_accumulate_divergence")
        for level in range(self.levels - 1, -1, -1):
            for _ in range(10):
                self.d.launch("k_dcgrid_jacobi", self.maxL[level], 64, self.g, C.c_uint8(level))
                self.d.launch("k_dcgrid_jacobi_inv", self.maxL[level], 64, self.g, C.c_uint8(level))
        self.d.launch("k_dcgrid_apply_pressure", self.B, 64, self.g)
        self._accumulate("k_dcgrid_accumulate_velocity")
        self.d.sync()

    def advectDensity(self):
        self.d.launch("k_dcgrid_advect_density", self.B, 64, self.g)
        N = self.numCells
        self.buf["density"][: 4 * N].copy_(self.buf["temporary"][: 4 * N])
        self._accumulate("k_dcgrid_accumulate_density")
        self.d.sync()

    # -- adaptTopology (cu:320-346) with the host ranking of cu:348-483
    def adaptTopology(self):
        self.d.launch("k_dcgrid_calc_vorticity", self.B, 64, self.g)
        touched = self.moveBlocks(0)
        if touched > 0:
            self._memset("hashKey", 0xFF)
            self._memset("hashVal", 0xFF)
            self.d.launch("k_dcgrid_refill_hash_table", self.gridSize, 256, self.g)
        touched = self.refineSubblocks(touched)
        if touched > 0:
            self.d.launch("k_dcgrid_refresh_apron_indices", self.B, 216, self.g)
            for level in range(self.levels - 2, -1, -1):
                self.d.launch("k_dcgrid_propagate_values", touched, 64, self.g, self.buf["touched"].data_ptr(),
                              C.c_int(level))
        self.d.sync()
        self.last_touched = touched

    def moveBlocks(self, touched):
        B = self.B
        self.d.launch("k_dcgrid_calc_subblock_scores", idiv_up(8 * B, 64), 64, self.g, self.buf["subScores"].data_ptr())
        self.d.launch("k_dcgrid_accumulate_subblock_scores", idiv_up(B, 64), 64, self.g,
                      self.buf["blockScores"].data_ptr(), self.buf["subScores"].data_ptr())
        self.d.sync()
        ss = self._d2h("subScores", np.float32, 8 * B)
        bs = self._d2h("blockScores", np.float32, B)
        self._memset("blockFlags", 0)
        loads = self._d2h("blockLoads", np.uint64, self.levels).astype(np.int64)
        moves, dests = [], []
        for level in range(self.levels - 1):
            d0, d1 = self.maxL[level], 8 * self.maxL[level + 1]
            l = min(d0, d1, int(loads[level]), self.full[level] - int(loads[level]))
            if self.moveLimit[level] > 0:
                l = min(l, self.moveLimit[level])
            if l == 0:
                continue
            mc = np.arange(self.off[level], self.off[level] + d0)
            neg = bs[mc] < 0
            mc = mc[np.lexsort((mc, np.where(neg, np.float32(np.inf), bs[mc]), neg))]
            dc = np.arange(8 * self.off[level + 1], 8 * self.off[level + 1] + d1)
            dc = dc[np.lexsort((dc, -ss[dc].astype(np.float64)))]
            matches = 0
            while (matches < l and bs[mc[matches]] >= 0 and ss[dc[matches]] >= 0
                   and bs[mc[matches]] < ss[dc[matches]]):
                matches += 1
                if matches < d1:
                    bs[dc[matches] // 8] = -FLT_MAX
            self.moveLimit[level] = int(np.float32(matches) * np.float32(1.2))
            moves += list(mc[:matches])
            dests += list(dc[:matches])
        n = len(moves)
        if n > 0:
            self._h2d("blockIdx", np.array(moves, np.uint64))
            self._h2d("destIdx", np.array(dests, np.uint64))
            self.d.launch("k_dcgrid_move_blocks", self.gridSize, 256, self.g, self.buf["blockIdx"].data_ptr(),
                          self.buf["destIdx"].data_ptr(), C.c_uint64(n))
            self.d.sync()
            self._h2d("touched", np.array(moves, np.uint64))
        self.last_moves = np.stack([np.array(moves, np.int64), np.array(dests, np.int64)], 1) if n else \
            np.zeros((0, 2), np.int64)
        return touched + n

    def refineSubblocks(self, touched):
        B = self.B
        self.d.launch("k_dcgrid_calc_subblock_scores", idiv_up(8 * B, 64), 64, self.g, self.buf["subScores"].data_ptr())
        self.d.sync()
        ss = self._d2h("subScores", np.float32, 8 * B)
        loads = self._d2h("blockLoads", np.uint64, self.levels)
        out = []
        for level in range(1, self.levels):
            a = np.uint64(self.maxL[level - 1]) - loads[level - 1]
            b = np.uint64(8) * loads[level] - loads[level - 1]
            limit = int(min(a, b))
            if limit == 0:
                continue
            s0 = 8 * self.off[level]
            cand = np.arange(s0, s0 + 8 * self.maxL[level])
            cand = cand[ss[cand] > np.float32(1e-4)]
            if len(cand) > limit:
                cand = cand[len(cand) - limit:]
            out += list(cand)
        n = len(out)
        self.last_refined = np.array(out, np.int64)
        if n > 0:
            self._h2d("destIdx", np.array(out, np.uint64))
            self.d.launch("k_dcgrid_refine_subblocks", idiv_up(n, 256), 256, self.g, self.buf["destIdx"].data_ptr(),
                          C.c_uint64(n), C.c_uint64(touched), self.buf["touched"].data_ptr())
            self.d.sync()
        return touched + n

    def step(self, n=1):
        for _ in range(n):
            self.advectVelocity()
            self.adaptTopology()
            self.project()
            self.advectDensity()

    # -- state read-out in the canonical layout of the oracle / product
    def snapshot(self):
        B, N = self.B, self.numCells
        pos = self._d2h("blockPositions", np.int32, 3 * B).reshape(B, 3)
        lvl = self._d2h("blockLevels", np.uint8, B)
        vel = self._d2h("velocity", np.float32, 3 * N).reshape(N, 3)
        tmp = self._d2h("temporary", np.float32, 3 * N)
        return dict(
            pos=pos, level=lvl, flags=self._d2h("blockFlags", np.uint8, B),
            parent=self._d2h("parentIndices", np.uint64, B).astype(np.int64),
            child=self._d2h("childIndices", np.uint64, 8 * B).astype(np.int64),
            apron=self._d2h("cellIndices", np.uint64, 216 * B).astype(np.int64),
            load=self._d2h("blockLoads", np.uint64, self.levels).astype(np.int64),
            move_limit=np.array(self.moveLimit, np.int64),
            density=self._d2h("density", np.float32, N), vel_x=vel[:, 0].copy(), vel_y=vel[:, 1].copy(),
            vel_z=vel[:, 2].copy(), fluidity=self._d2h("fluidity", np.float32, N),
            divergence=tmp[:N].copy(), pressure=tmp[N:2 * N].copy(), pressure_tmp=tmp[2 * N:3 * N].copy())

    def apply_decisions(self, moves, refines):
        """adaptTopology (cu:320-346) with the candidate lists given instead of
        ranked: moves = (block, destination subblock) pairs, refines = subblocks."""
        self.d.launch("k_dcgrid_calc_vorticity", self.B, 64, self.g)
        self._memset("blockFlags", 0)
        touched = 0
        n = len(moves)
        if n:
            self._h2d("blockIdx", np.array([m[0] for m in moves], np.uint64))
            self._h2d("destIdx", np.array([m[1] for m in moves], np.uint64))
            self.d.launch("k_dcgrid_move_blocks", self.gridSize, 256, self.g, self.buf["blockIdx"].data_ptr(),
                          self.buf["destIdx"].data_ptr(), C.c_uint64(n))
            self.d.sync()
            self._h2d("touched", np.array([m[0] for m in moves], np.uint64))
            touched = n
            self._memset("hashKey", 0xFF)
            self._memset("hashVal", 0xFF)
            self.d.launch("k_dcgrid_refill_hash_table", self.gridSize, 256, self.g)
        r = len(refines)
        if r:
            self._h2d("destIdx", np.array(refines, np.uint64))
            self.d.launch("k_dcgrid_refine_subblocks", idiv_up(r, 256), 256, self.g, self.buf["destIdx"].data_ptr(),
                          C.c_uint64(r), C.c_uint64(touched), self.buf["touched"].data_ptr())
            touched += r
        if touched:
            self.d.launch("k_dcgrid_refresh_apron_indices", self.B, 216, self.g)
            for level in range(self.levels - 2, -1, -1):
                self.d.launch("k_dcgrid_propagate_values", touched, 64, self.g, self.buf["touched"].data_ptr(),
                              C.c_int(level))
        self.d.sync()


class UniformGridStruct(C.Structure):
    """struct UniformGrid (src/uniformgrid/uniformgrid.h:31-46)"""
    _fields_ = [(n, C.c_uint64) for n in ["density", "velocity", "fluidity", "pressure", "temporary",
                                          "t_velocity", "t_pressure", "divergence", "t_density"]]


class RefUniform:
    """FluidSimulationUniform (fluid_simulation_uniform.cu:6-176) over the
    reference's uniform-grid kernels."""

    def __init__(self, drv, params):
        import torch
        self.d, self.t, self.p = drv, torch, params
        size = (params.gx, params.gy, params.gz)
        minDim = min(size)
        cellSize, lv = 2, 1
        while all(s % cellSize == 0 for s in size) and cellSize * 4 <= minDim:
            lv += 1
            cellSize *= 2
        self.levels = lv
        bs = (8, 8, 4)
        self.blockSize = bs
        self.gridSize = tuple(idiv_up(size[i], bs[i]) for i in range(3))
        ms = list(size)
        self.bsl, self.gsl = [], []
        for _ in range(lv):
            b = tuple(min(bs[i], ms[i]) for i in range(3))
            self.bsl.append(b)
            self.gsl.append(tuple(idiv_up(ms[i], b[i]) for i in range(3)))
            ms = [m // 2 for m in ms]
        self.numCells = size[0] * size[1] * size[2]
        s, mip = 1, 0
        while all(x % s == 0 for x in size):
            mip += self.numCells // (s * s * s)
            s *= 2
        self.mip = mip
        N = self.numCells
        u8 = lambda n: torch.zeros(max(int(n), 16), dtype=torch.uint8, device="cuda")
        self.buf = dict(density=u8(4 * N), velocity=u8(12 * N), pressure=u8(4 * mip), fluidity=u8(4 * mip),
                        temporary=u8(12 * N))
        self.h = UniformGridStruct()
        for n in ["density", "velocity", "fluidity", "pressure", "temporary"]:
            setattr(self.h, n, self.buf[n].data_ptr())
        raw = bytes(self.h)
        self.d_grid = u8(len(raw))
        self.d_grid[: len(raw)].copy_(torch.frombuffer(bytearray(raw), dtype=torch.uint8))
        sp = sim_params_from(params)
        ptr, sz = drv.global_ptr("params")
        drv._chk(drv.cu.cuMemcpyHtoD_v2(C.c_uint64(ptr), C.byref(sp), C.c_size_t(sz)), "params")
        self.d.launch("k_uniform_init_aliasses", 1, 1, self.g)
        self.d.sync()
        self.reset()

    @property
    def g(self):
        return self.d_grid.data_ptr()

    def reset(self):
        for n in ["density", "velocity", "pressure", "fluidity"]:
            self.buf[n].fill_(0)
        self.adaptTopology()
        self.d.launch("k_uniform_init", self.gridSize, self.blockSize, self.g)
        self.d.sync()

    def adaptTopology(self):
        for l in range(self.levels):
            self.d.launch("k_uniform_set_solidity_ratio", self.gsl[l], self.bsl[l], self.g, C.c_int(l))
        self.d.sync()

    def advectVelocity(self):
        self.d.launch("k_uniform_advect_velocity", self.gridSize, self.blockSize, self.g)
        self.buf["velocity"].copy_(self.buf["temporary"])
        self.d.sync()

    def _jacobi(self, level, pairs):
        for _ in range(pairs):
            self.d.launch("k_uniform_jacobi", self.gsl[level], self.bsl[level], self.g, C.c_int(level))
            self.d.launch("k_uniform_jacobi_inv", self.gsl[level], self.bsl[level], self.g, C.c_int(level))

    def project(self):
        self.d.launch("k_uniform_calc_divergence", self.gridSize, self.blockSize, self.g)
        for l in range(1, self.levels):
            self.d.launch("k_uniform_restrict", self.gsl[l], self.bsl[l], self.g, C.c_int(l))
        self._jacobi(self.levels - 1, 2)
        for l in range(self.levels - 2, -1, -1):
            self.d.launch("k_uniform_prolongate", self.gsl[l], self.bsl[l], self.g, C.c_int(l))
            self._jacobi(l, 1)
        self.d.launch("k_uniform_apply_pressure", self.gridSize, self.blockSize, self.g)
        self.d.sync()

    def projectLocal(self):
        self.d.launch("k_uniform_calc_divergence", self.gridSize, self.blockSize, self.g)
        self._jacobi(0, 5)
        self.d.launch("k_uniform_apply_pressure", self.gridSize, self.blockSize, self.g)
        self.d.sync()

    def advectDensity(self):
        self.d.launch("k_uniform_advect_density", self.gridSize, self.blockSize, self.g)
        self.buf["density"][: 4 * self.numCells].copy_(self.buf["temporary"][: 4 * self.numCells])
        self.d.sync()

    def step(self, n=1):
        for _ in range(n):
            self.advectVelocity()
            self.adaptTopology()
            self.project()
            self.advectDensity()

    def snapshot(self):
        N, mip = self.numCells, self.mip
        f = lambda name, n: self.buf[name][: 4 * n].cpu().numpy().view(np.float32).copy()
        vel = self.buf["velocity"].cpu().numpy().view(np.float32).reshape(N, 3)
        tmp = self.buf["temporary"].cpu().numpy().view(np.float32)
        return dict(density=f("density", N), vel_x=vel[:, 0].copy(), vel_y=vel[:, 1].copy(),
                    vel_z=vel[:, 2].copy(), fluidity=f("fluidity", N), pressure=f("pressure", N),
                    pressure_tmp=tmp[:N].copy(), divergence=tmp[mip:mip + N].copy())
