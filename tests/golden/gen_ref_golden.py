"""Generates the golden fixtures of tests/golden/ from the reference's own CUDA
kernels (oracle/_ref/*.cubin, built by oracle/build_ref.sh from the reference
sources) on a GPU:

    python tests/golden/gen_ref_golden.py OUT_DIR

Adaptive cases (small domains, reference defaults):
  init0..init5   state before and after each of the 5 adaptTopology passes of
                 init() (fluid_simulation_dcgrid.cu:207-209): refinement,
                 apron refresh, value propagation
  s0..s5         after 2 steps: state before advectVelocity, after it, after
                 adaptTopology, project, advectDensity, and after projectLocal
  replay_pre / replay_post / replay_moves
                 block moves chosen by the oracle's non-compat selection and
                 applied with the reference's move, hash-refill, apron-refresh
                 and propagation kernels
Uniform cases: u0..u5, the same stage sequence on the uniform grid.
Fixtures store block tables as int32 and fields as float32.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

TOPO = ("pos", "level", "parent", "child", "apron", "load", "move_limit")
FIELDS = ("density", "vel_x", "vel_y", "vel_z", "fluidity", "divergence", "pressure", "pressure_tmp")


def pack(snap, label, out, with_topo=True):
    for k, v in snap.items():
        if k in TOPO and not with_topo:
            continue
        if k in ("parent", "child", "apron"):
            v = v.astype(np.int32)
        elif k == "pos":
            v = v.astype(np.int32)
        out[f"{label}__{k}"] = v


def params_json(p):
    from dcgrid_gb300 import capi
    return np.array(json.dumps(capi.params_to_dict(p)))


def adaptive_case(drv, p, replay=False):
    from oracle import ref_driver
    from oracle.pyoracle import OracleSim
    from dcgrid_gb300 import capi
    out = {"params": params_json(p)}
    r = ref_driver.RefDCGrid(drv, p, init_passes=0)
    pack(r.snapshot(), "init0", out)
    for i in range(5):
        r.adaptTopology()
        pack(r.snapshot(), f"init{i + 1}", out)
    r.step(2)
    pack(r.snapshot(), "s0", out)
    r.advectVelocity()
    pack(r.snapshot(), "s1", out)
    r.adaptTopology()
    pack(r.snapshot(), "s2", out)
    r.project()
    pack(r.snapshot(), "s3", out)
    r.advectDensity()
    pack(r.snapshot(), "s4", out)
    r.projectLocal()
    pack(r.snapshot(), "s5", out)
    if replay:
        # decisions of the non-compat selection, taken by the oracle from the
        # reference's current state, then applied with the reference's kernels
        pre = r.snapshot()
        q = capi.params_from_dict(capi.params_to_dict(p))
        q.ref_compat = 0
        q.init_adapt_passes = 0
        o = OracleSim(q, precision="float")
        load_oracle(o, pre)
        o.adapt()
        moves, refines = o.get_last_adapt()
        assert len(refines) == 0, "replay case expects moves only"
        r.apply_decisions([tuple(m) for m in moves], [])
        pack(pre, "replay_pre", out)
        pack(r.snapshot(), "replay_post", out)
        out["replay_moves"] = moves.astype(np.int64)
    return out


def load_oracle(o, snap):
    """Loads a reference snapshot (block table, apron table, fields) into an oracle."""
    B = snap["pos"].shape[0]
    pos = np.zeros((B, 4), np.int32)
    pos[:, :3] = snap["pos"]
    pos[:, 3] = np.where(snap["level"] == 255, -1, snap["level"].astype(np.int32))
    to_u32 = lambda a: np.where(np.asarray(a) < 0, 0xFFFFFFFF, np.asarray(a)).astype(np.uint32)
    o.set_topology(dict(pos=pos, parent=to_u32(snap["parent"]), child=to_u32(snap["child"]).reshape(B, 8),
                        load=snap["load"], move_limit=snap["move_limit"]))
    o.set_apron(np.asarray(snap["apron"], np.int64).reshape(B, 216))
    for f in FIELDS:
        o.set_field(f, np.asarray(snap[f], np.float64))


def uniform_case(drv, p):
    from oracle import ref_driver
    out = {"params": params_json(p)}
    r = ref_driver.RefUniform(drv, p)
    r.step(2)
    pack(r.snapshot(), "u0", out)
    r.advectVelocity()
    pack(r.snapshot(), "u1", out)
    r.adaptTopology()
    pack(r.snapshot(), "u2", out)
    r.project()
    pack(r.snapshot(), "u3", out)
    r.advectDensity()
    pack(r.snapshot(), "u4", out)
    r.projectLocal()
    pack(r.snapshot(), "u5", out)
    return out


def main(out_dir):
    from oracle import ref_driver
    from tests import scenarios
    os.makedirs(out_dir, exist_ok=True)
    drv = ref_driver.Driver(os.path.join(ref_driver.REF_DIR, "ref_dcgrid.cubin"))
    cases = {
        "ref_default_16x32x16_b80": (scenarios.ref_default(16, 32, 16, 80), False),
        "ref_sphere_16x32x16_b80": (scenarios.sphere_obstacle(16, 32, 16, 80), False),
        "ref_default_32x32x32_b120": (scenarios.ref_default(32, 32, 32, 120), True),
    }
    for name, (p, replay) in cases.items():
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **adaptive_case(drv, p, replay))
        print("wrote", name, flush=True)
    udrv = ref_driver.Driver(os.path.join(ref_driver.REF_DIR, "ref_uniform.cubin"))
    ucases = {
        "uniform_default_16x32x16": scenarios.ref_default(16, 32, 16, 0),
        "uniform_sphere_16x32x16": scenarios.sphere_obstacle(16, 32, 16, 0),
    }
    for name, p in ucases.items():
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **uniform_case(udrv, p))
        print("wrote", name, flush=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "golden_out")
