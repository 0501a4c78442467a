"""Pins the oracle to the reference itself: golden fixtures produced by the
reference's own CUDA kernels (tests/golden/gen_ref_golden.py, compiled from
the reference sources with -fmad=false) are loaded into the oracle's float
mirror, one stage is run, and the result must equal the reference's output
bit for bit.

Refinements allocate blocks through atomicAdd in the reference
(dcgrid_utils.cuh:118), so the index a new block gets there depends on thread
timing; after an adaptation, blocks are matched by (level, position) and
block/cell indices are compared through that matching.
"""
import glob
import json
import os

import numpy as np
import pytest

from dcgrid_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
FIELDS = ("density", "vel_x", "vel_y", "vel_z", "fluidity", "divergence", "pressure", "pressure_tmp")

pytestmark = pytest.mark.usefixtures("oracle_lib")


def load(path):
    z = np.load(path)
    params = capi.params_from_dict(json.loads(str(z["params"])))
    snaps = {}
    for k in z.files:
        if "__" in k:
            label, name = k.split("__", 1)
            snaps.setdefault(label, {})[name] = z[k]
    return params, snaps, z


def oracle_from(params, snap, mode=capi.MODE_ADAPTIVE, compat=None):
    from oracle.pyoracle import OracleSim
    q = capi.params_from_dict(capi.params_to_dict(params))
    q.init_adapt_passes = 0
    if compat is not None:
        q.ref_compat = compat
    o = OracleSim(q, mode=mode, precision="float")
    if mode == capi.MODE_ADAPTIVE:
        B = snap["pos"].shape[0]
        pos = np.zeros((B, 4), np.int32)
        pos[:, :3] = snap["pos"]
        pos[:, 3] = np.where(snap["level"] == 255, -1, snap["level"].astype(np.int32))
        u32 = lambda a: np.where(np.asarray(a, np.int64) < 0, 0xFFFFFFFF, np.asarray(a, np.int64)).astype(np.uint32)
        o.set_topology(dict(pos=pos, parent=u32(snap["parent"]), child=u32(snap["child"]).reshape(B, 8),
                            load=snap["load"], move_limit=snap["move_limit"]))
        o.set_apron(np.asarray(snap["apron"], np.int64).reshape(B, 216))
    for f in FIELDS:
        if f in snap:
            o.set_field(f, np.asarray(snap[f], np.float64))
    return o


def oracle_state(o):
    t = o.get_topology()
    i64 = lambda a: np.where(a == 0xFFFFFFFF, -1, a.astype(np.int64))
    st = dict(pos=t["pos"][:, :3], level=np.where(t["pos"][:, 3] < 0, 255, t["pos"][:, 3]),
              parent=i64(t["parent"]), child=i64(t["child"].reshape(-1)), apron=o.get_apron().reshape(-1),
              load=t["load"])
    for f in FIELDS:
        st[f] = o.get_field(f).astype(np.float32)
    return st


def block_map(g, o):
    """golden block index -> oracle block index, matched by (level, position)."""
    def keys(s):
        return {(int(l), int(p[0]), int(p[1]), int(p[2])): i
                for i, (p, l) in enumerate(zip(s["pos"], s["level"])) if l != 255}
    gk, ok = keys(g), keys(o)
    assert set(gk) == set(ok), f"block sets differ: {len(set(gk) ^ set(ok))} blocks"
    m = np.full(len(g["pos"]), -1, np.int64)
    for k, i in gk.items():
        m[i] = ok[k]
    return m


def compare_adaptive(g, o, fields, topo=True):
    m = block_map(g, o)
    alloc = np.nonzero(m >= 0)[0]
    if topo:
        assert np.array_equal(np.asarray(g["load"]), np.asarray(o["load"])), "loads differ"
        gp = np.asarray(g["parent"])[alloc]
        mp = np.where(gp < 0, -1, m[np.maximum(gp, 0) // 8] * 8 + np.maximum(gp, 0) % 8)
        assert np.array_equal(mp, o["parent"][m[alloc]]), "parents differ"
        gc = np.asarray(g["child"]).reshape(-1, 8)[alloc]
        mc = np.where(gc < 0, -1, m[np.maximum(gc, 0)])
        assert np.array_equal(mc, o["child"].reshape(-1, 8)[m[alloc]]), "children differ"
        ga = np.asarray(g["apron"], np.int64).reshape(-1, 216)[alloc]
        ma = m[ga // 64] * 64 + ga % 64
        oa = o["apron"].reshape(-1, 216)[m[alloc]]
        assert np.array_equal(ma, oa), f"apron entries differ in {(ma != oa).sum()} places"
    cells_g = (alloc[:, None] * 64 + np.arange(64)).reshape(-1)
    cells_o = (m[alloc][:, None] * 64 + np.arange(64)).reshape(-1)
    for f in fields:
        a = np.asarray(g[f], np.float32)[cells_g]
        b = o[f][cells_o]
        bad = a != b
        assert not bad.any(), f"{f}: {bad.sum()} of {bad.size} cells differ, max |d| " \
                              f"{np.abs(a.astype(np.float64) - b)[bad].max():.3g}"


ADAPTIVE = [f for f in FIXTURES if not os.path.basename(f).startswith("uniform")]
UNIFORM = [f for f in FIXTURES if os.path.basename(f).startswith("uniform")]


def test_fixtures_present():
    assert len(ADAPTIVE) >= 3 and len(UNIFORM) >= 1, "golden fixtures missing (tests/golden/*.npz)"


@pytest.mark.parametrize("path", ADAPTIVE, ids=os.path.basename)
def test_init_adaptation_passes(path):
    """The 5 adaptTopology passes of init(): refinement, apron refresh, propagation."""
    params, snaps, _ = load(path)
    for k in range(5):
        o = oracle_from(params, snaps[f"init{k}"])
        o.adapt()
        compare_adaptive(snaps[f"init{k + 1}"], oracle_state(o), ("density", "vel_x", "vel_y", "vel_z", "fluidity"))


STAGES = [("s0", "advect_velocity", "s1", ("vel_x", "vel_y", "vel_z")),
          ("s1", "adapt", "s2", ("density", "vel_x", "vel_y", "vel_z", "fluidity")),
          ("s2", "project", "s3", ("vel_x", "vel_y", "vel_z", "pressure", "pressure_tmp", "divergence")),
          ("s3", "advect_scalars", "s4", ("density",)),
          ("s4", "project_local", "s5", ("vel_x", "vel_y", "vel_z", "pressure", "pressure_tmp", "divergence"))]


@pytest.mark.parametrize("path", ADAPTIVE, ids=os.path.basename)
@pytest.mark.parametrize("stage", STAGES, ids=lambda s: s[1])
def test_stage_matches_reference(path, stage):
    params, snaps, _ = load(path)
    before, fn, after, fields = stage
    o = oracle_from(params, snaps[before])
    getattr(o, fn)()
    compare_adaptive(snaps[after], oracle_state(o), fields, topo=(fn == "adapt"))


@pytest.mark.parametrize("path", [p for p in ADAPTIVE if "replay_pre__pos" in np.load(p).files],
                         ids=os.path.basename)
def test_block_moves_match_reference(path):
    """Moves applied with the reference's move / hash-refill / refresh /
    propagation kernels equal the oracle's replay of the same decisions."""
    params, snaps, z = load(path)
    moves = z["replay_moves"]
    assert len(moves) > 0
    o = oracle_from(params, snaps["replay_pre"], compat=1)
    o.adapt_replay(moves, np.zeros((0, 2), np.int64))
    compare_adaptive(snaps["replay_post"], oracle_state(o), ("density", "vel_x", "vel_y", "vel_z", "fluidity"))


USTAGES = [("u0", "advect_velocity", "u1", ("vel_x", "vel_y", "vel_z")),
           ("u1", "adapt", "u2", ("fluidity",)),
           ("u2", "project", "u3", ("vel_x", "vel_y", "vel_z", "pressure", "pressure_tmp", "divergence")),
           ("u3", "advect_scalars", "u4", ("density",)),
           ("u4", "project_local", "u5", ("vel_x", "vel_y", "vel_z", "pressure", "pressure_tmp", "divergence"))]


@pytest.mark.parametrize("path", UNIFORM, ids=os.path.basename)
@pytest.mark.parametrize("stage", USTAGES, ids=lambda s: s[1])
def test_uniform_stage_matches_reference(path, stage):
    params, snaps, _ = load(path)
    before, fn, after, fields = stage
    o = oracle_from(params, snaps[before], mode=capi.MODE_UNIFORM)
    getattr(o, fn)()
    for f in fields:
        a = np.asarray(snaps[after][f], np.float32)
        b = o.get_field(f).astype(np.float32)
        bad = a != b
        assert not bad.any(), f"{f}: {bad.sum()} cells differ"
