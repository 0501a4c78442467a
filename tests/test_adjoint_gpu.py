"""Adjoint of the density path on the GPU (an extension without reference counterpart).

* state save/load reproduces a run exactly (checkpoints of the adjoint);
* the GPU adjoint is the transpose of the GPU step (dot-product tests) and
  agrees with the FP64 host adjoint of the oracle on the same state;
* the 32-step rollout on an effective 128^3 2-level grid, differentiated with
  respect to the 16^3 emission map through a torch.autograd.Function over the
  C ABI (checkpoints every 8 steps, recomputation), matches central finite
  differences (eps = 1e-3) along 8 seeded directions and the FP64 host
  adjoint of the same rollout, both within 1e-3 relative.
"""
import ctypes as C

import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib", "oracle_lib")]

STEPS, EVERY, EM_N = 32, 8, 16


def gpu(p):
    from dcgrid_gb300 import Simulation
    return Simulation(p)


def cells_of(s):
    return np.repeat(s.get_topology()["pos"][:, 3] >= 0, 64)


def test_state_roundtrip_is_exact(tmp_path):
    import torch
    p = scenarios.cloud(64, 1500, 3, 10, 0)
    s = gpu(p)
    s.add_velocity_noise(3, 0.5)
    s.step(3)
    host = s.save_state()
    dev = s.save_state(torch.empty(s.state_bytes(), dtype=torch.uint8, device="cuda"))
    s.save(str(tmp_path / "state.bin"))
    s.step(4)
    ref = {f: s.get_field(f) for f in ["density", "temperature", "vel_x", "pressure"]}
    topo = s.get_topology()
    for restore in [lambda: s.load_state(host), lambda: s.load_state(dev), lambda: s.load(str(tmp_path / "state.bin"))]:
        restore()
        s.step(4)
        for f, v in ref.items():
            assert np.array_equal(s.get_field(f), v), f
        assert np.array_equal(s.get_topology()["pos"], topo["pos"])
    other = gpu(scenarios.cloud(64, 1400, 3, 10, 0))
    with pytest.raises(Exception):
        other.load_state(host)


def adj_gpu(s, lam, lam_em=None):
    import torch
    li = torch.from_numpy(np.ascontiguousarray(lam, np.float32)).cuda()
    lo = torch.empty_like(li)
    s.adjoint_step(li, lo, lam_em)
    torch.cuda.synchronize()
    return lo.cpu().numpy().astype(np.float64)


def test_gpu_adjoint_is_the_transpose_of_the_gpu_step():
    import torch
    p = scenarios.differentiable(32, 3, iters=10, em_n=8)
    em = scenarios.emission_field(8, 3)
    s = gpu(p)
    s.set_emission(em)
    s.add_velocity_noise(0, 0.5)
    s.step(3)
    base = s.save_state()
    rng = np.random.default_rng(4)
    cells = cells_of(s)
    dq = np.where(cells, rng.standard_normal(cells.size), 0.0).astype(np.float32)
    s.set_field("density", s.get_field("density") + dq)
    s.step(1)
    qb = s.get_field("density").astype(np.float64)
    s.load_state(base)
    s.step(1)
    qa = s.get_field("density").astype(np.float64)
    st = s.stats()
    assert st.moved_blocks + st.refined_subblocks > 0
    lam = np.where(cells_of(s), rng.standard_normal(cells.size), 0.0)
    lam_em = torch.zeros(8 ** 3, device="cuda")
    jt = adj_gpu(s, lam, lam_em)
    lhs, rhs = float(lam @ (qb - qa)), float(jt @ dq.astype(np.float64))
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs), (lhs, rhs)
    # emission direction
    de = rng.standard_normal(em.size).astype(np.float32)
    s.load_state(base)
    s.set_emission(em + de)
    s.step(1)
    qe = s.get_field("density").astype(np.float64)
    lhs, rhs = float(lam @ (qe - qa)), float(lam_em.cpu().numpy().astype(np.float64) @ de)
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs), (lhs, rhs)


def test_gpu_adjoint_matches_fp64_host_adjoint():
    import torch
    from oracle.pyoracle import OracleSim
    p = scenarios.differentiable(32, 3, iters=10, em_n=8)
    em = scenarios.emission_field(8, 3)
    g, o = gpu(p), OracleSim(p, precision="double")
    for s in (g, o):
        s.set_emission(em)
        s.add_velocity_noise(0, 0.5)
    for _ in range(4):
        g.advect_velocity(); o.advect_velocity()
        g.adapt()
        mv, rf = g.get_last_adapt()
        o.adapt_replay(mv, rf)
        g.project(); o.project()
        g.advect_scalars(); o.advect_scalars()
    g.sync()
    assert len(mv) > 0  # the last step moved blocks: propagation transpose exercised
    rng = np.random.default_rng(5)
    lam = np.where(cells_of(g), rng.standard_normal(64 * p.max_blocks), 0.0)
    lam_em_g = torch.zeros(8 ** 3, device="cuda")
    lam_em_o = np.zeros(8 ** 3)
    jg = adj_gpu(g, lam, lam_em_g)
    jo = o.adjoint_step(lam, lam_em_o)
    assert np.linalg.norm(jg - jo) <= 1e-4 * np.linalg.norm(jo)
    eg = lam_em_g.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(eg - lam_em_o) <= 1e-4 * np.linalg.norm(lam_em_o)


# ---------------------------------------------------------------- rollout
def dense_density(s):
    import torch
    p = s.params
    out = torch.empty(p.gx * p.gy * p.gz, dtype=torch.float32, device="cuda")
    rc = s.L.dcg_get_dense(s.h, capi.FIELD_DENSITY, C.c_void_p(out.data_ptr()), capi.DEVICE)
    assert rc == 0
    s.sync()
    return out


def make_rollout():
    import torch

    class Rollout(torch.autograd.Function):
        """STEPS steps from a saved initial state with emission map E; returns
        the dense density. Backward: the transposed steps in reverse, each
        step's state recomputed from the checkpoint every EVERY steps."""

        @staticmethod
        def forward(ctx, E, sim, state0):
            sim.load_state(state0)
            sim.set_emission(E.detach().contiguous())
            ckpt = {0: state0}
            for t in range(1, STEPS + 1):
                sim.step(1)
                if t % EVERY == 0 and t < STEPS:
                    ckpt[t] = sim.save_state(torch.empty_like(state0))
            ctx.sim, ctx.ckpt = sim, ckpt
            return dense_density(sim)

        @staticmethod
        def backward(ctx, g_rho):
            sim, ckpt = ctx.sim, ctx.ckpt
            ncell = 64 * sim.params.max_blocks
            lam = torch.zeros(ncell, device="cuda")
            sim.adjoint_dense(g_rho.contiguous(), lam)  # sim holds the final state
            lam_e = torch.zeros(EM_N ** 3, device="cuda")
            nxt = torch.empty_like(lam)
            for t in range(STEPS, 0, -1):
                seg = (t - 1) // EVERY * EVERY
                sim.load_state(ckpt[seg])
                sim.step(t - seg)
                sim.adjoint_step(lam, nxt, lam_e)
                lam, nxt = nxt, lam
            torch.cuda.synchronize()
            return lam_e, None, None

    return Rollout


@pytest.fixture(scope="module")
def config4():
    import torch
    p = scenarios.differentiable(128, 2, iters=20, em_n=EM_N)
    s = gpu(p)
    s.add_velocity_noise(0, 0.5)
    state0 = s.save_state(torch.empty(s.state_bytes(), dtype=torch.uint8, device="cuda"))
    Rollout = make_rollout()
    E_t = torch.from_numpy(scenarios.emission_field(EM_N, 1)).cuda()
    with torch.no_grad():
        target = Rollout.apply(E_t, s, state0).clone()
    E0 = torch.from_numpy(scenarios.emission_field(EM_N, 0)).cuda().requires_grad_(True)

    def loss_of(E):
        return ((Rollout.apply(E, s, state0).double() - target.double()) ** 2).sum()

    L = loss_of(E0)
    L.backward()
    return dict(p=p, sim=s, state0=state0, target=target, E0=E0, grad=E0.grad.detach().double().clone(),
                loss_of=loss_of)


def test_config4_gradient_matches_central_differences(config4):
    import torch
    g, E0, loss_of = config4["grad"], config4["E0"].detach(), config4["loss_of"]
    eps = 1e-3
    rng = np.random.default_rng(8)
    errs = []
    for _ in range(8):
        d = torch.from_numpy(rng.standard_normal(EM_N ** 3).astype(np.float32)).cuda()
        with torch.no_grad():
            fd = (loss_of(E0 + eps * d) - loss_of(E0 - eps * d)).item() / (2 * eps)
        an = float((g * d.double()).sum())
        errs.append(abs(fd - an) / max(abs(fd), 1e-30))
    print("central-difference relative errors:", [f"{e:.2e}" for e in errs])
    assert max(errs) <= 1e-3, errs


def test_config4_gradient_matches_fp64_host_adjoint(config4):
    from oracle.pyoracle import OracleSim, set_threads
    import os
    set_threads(os.cpu_count() or 1)
    p, s = config4["p"], config4["sim"]
    E0 = config4["E0"].detach().cpu().numpy().astype(np.float64)
    target = config4["target"].cpu().numpy().astype(np.float64)
    # the GPU run's adaptation decisions, step by step (stage calls)
    s.load_state(config4["state0"])
    s.set_emission(config4["E0"].detach().contiguous())
    decisions = []
    for _ in range(STEPS):
        s.advect_velocity()
        s.adapt()
        decisions.append(s.get_last_adapt())
        s.project()
        s.advect_scalars()
    o = OracleSim(p, precision="double")
    o.set_emission(E0)
    o.add_velocity_noise(0, 0.5)

    def step(sim, t):
        sim.advect_velocity()
        sim.adapt_replay(*decisions[t])
        sim.project()
        sim.advect_scalars()

    ckpt = {}
    for t in range(STEPS):
        if t % EVERY == 0:
            c = OracleSim(p, precision="double")
            c.copy_state_from(o)
            ckpt[t] = c
        step(o, t)
    rho = o.get_dense("density").reshape(-1)
    lam = np.zeros(64 * p.max_blocks)
    o.adjoint_dense(2.0 * (rho - target), lam)
    lam_e = np.zeros(EM_N ** 3)
    for t in range(STEPS, 0, -1):
        seg = (t - 1) // EVERY * EVERY
        o.copy_state_from(ckpt[seg])
        for k in range(seg, t):
            step(o, k)
        lam = o.adjoint_step(lam, lam_e)
    g = config4["grad"].cpu().numpy()
    rel = np.linalg.norm(g - lam_e) / np.linalg.norm(lam_e)
    print("GPU FP32 vs FP64 host adjoint gradient, relative L2:", f"{rel:.2e}")
    assert rel <= 1e-3, rel
