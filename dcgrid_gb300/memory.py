"""Memory-budget calculators.

`plan_bytes` / `blocks_for_budget` / `uniform_edge_for_budget` size this
library's layout exactly (dcg_plan_bytes, dcg_blocks_for_budget: no GPU
needed). `reference_*` restate the reference's own estimates for its layout
(scripts/calcMemoryAdaptiveGrid.js, calcMemoryUniformGrid.js,
calcActiveBlocks.js), for side-by-side budgets.
"""
import ctypes as C

from . import capi
from .sim import DcgError, lib


def _lib():
    L = lib()
    L.dcg_plan_bytes.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]
    L.dcg_blocks_for_budget.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
    return L


def plan_bytes(params, mode=capi.MODE_ADAPTIVE):
    """Device bytes dcg_create(params, mode) allocates."""
    n = C.c_int64()
    rc = _lib().dcg_plan_bytes(C.byref(params), mode, C.byref(n))
    if rc:
        raise DcgError(rc, "dcg_plan_bytes")
    return n.value


def blocks_for_budget(params, budget_bytes):
    """Largest block budget whose adaptive allocation fits budget_bytes, capped
    at the full block count of every level."""
    n = C.c_int64()
    rc = _lib().dcg_blocks_for_budget(C.byref(params), int(budget_bytes), C.byref(n))
    if rc:
        raise DcgError(rc, "dcg_blocks_for_budget")
    return n.value


def uniform_edge_for_budget(params, budget_bytes, multiple=64):
    """Largest cube edge (a multiple of `multiple`) whose uniform-grid
    allocation with params' scalars fits budget_bytes."""
    p = capi.params_from_dict(capi.params_to_dict(params))
    best, edge = 0, multiple
    while True:
        p.gx = p.gy = p.gz = edge
        if plan_bytes(p, capi.MODE_UNIFORM) > budget_bytes:
            return best
        best, edge = edge, edge + multiple


# ---- the reference's estimates for its own layout -----------------------------
def reference_adaptive_bytes(num_blocks, channels=12):
    """scripts/calcMemoryAdaptiveGrid.js:4-27: per level 12 size_t; per block a
    14 B header and 5 indices, 8 subblocks of 12 B + an index, 4 hash entries
    of 8 B + an index, 64 cells of 4*channels + 1 B, and a 216-entry index
    apron."""
    index = 8
    per_level = 12 * index
    per_block = (1 * (14 + 5 * index) + 8 * (12 + index) + 4 * (8 + index) + 64 * (4 * channels + 1)
                 + 216 * index)
    return per_level + num_blocks * per_block, per_block


def reference_uniform_bytes(w, h, d, channels=18):
    """scripts/calcMemoryUniformGrid.js:1-21: 4*channels + 1 B per cell plus
    4 B per cell of the coarser mip levels."""
    cells = w * h * d
    mip, s = 0, 1
    while w % s == 0 and h % s == 0 and d % s == 0:
        mip += cells // (s * s * s)
        s *= 2
    return cells * (4 * channels + 1) + (mip - cells) * 4


def reference_active_cells(total_blocks):
    """scripts/calcActiveBlocks.js:6-11: the root block gives 8 active
    subblocks and every further block 8 and takes one: 7n + 1 subblocks."""
    subblocks = 7 * total_blocks + 1
    return subblocks, 8 * subblocks
