"""Full adjoint of the step on the GPU (dcg_adjoint_step_full): velocity and
every scalar, buoyancy, the pressure projection as a transposed cascade, and
the dependence of the semi-Lagrangian sample positions on the velocity, with
the block topology recorded.

* one step: the GPU adjoint equals the FP64 host adjoint of the oracle on the
  same state (decisions replayed);
* a buoyant variant of the differentiable rollout (effective 128^3, 2 levels,
  100 Jacobi sweeps per level, temperature and density driving buoyancy with
  alpha = 0.1, beta = 0.3, a 16^3 emission map, 32 steps, checkpoints every 8
  steps with recomputation, torch.autograd.Function over the C ABI): the
  gradient of the density loss with respect to the emission map matches the
  FP64 host adjoint of the same rollout within 1e-3 relative, and FP32
  central differences (eps = 1e-3 along 8 seeded unit directions) within
  1e-2. With buoyancy the perturbed runs move sample points, and the
  semi-Lagrangian sample is not differentiable where a point crosses a level
  interface (injected coarse ghosts on one side, the coarse lattice on the
  other); FP32 differences over 32 steps pick up such crossings, which bounds
  their agreement. The FP64 host adjoint itself matches FP64 central
  differences of a buoyant rollout at eps = 1e-6 to 1e-5
  (tests/test_adjoint_full_oracle.py).
"""
import ctypes as C

import numpy as np
import pytest

from dcgrid_gb300 import capi
from tests import scenarios

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("cuda_ok", "dcg_lib", "oracle_lib")]

STEPS, EVERY, EM_N = 32, 8, 16


def buoyant(g=128, levels=2, iters=100, em_n=EM_N):
    """The differentiable scene with temperature and buoyancy: a hot sphere
    (temperature 10, no density) near the bottom centre and the emission map's
    density, alpha = 0.1, beta = 0.3."""
    p = scenarios.differentiable(g, levels, iters=iters, em_n=em_n)
    p.n_scalars = 3
    p.buoy_alpha = 0.1
    p.buoy_beta = 0.3
    p.t_ambient = 0.0
    p.src_enabled = 1
    p.src_center[0] = g / 2.0
    p.src_center[1] = g / 8.0
    p.src_center[2] = g / 2.0
    p.src_radius = g / 16.0
    p.src_density = 0.0
    p.src_temperature = 10.0
    p.src_vapor = 0.0
    return p


def test_one_step_full_adjoint_matches_fp64_host_adjoint():
    import torch
    from dcgrid_gb300 import Simulation
    from oracle.pyoracle import OracleSim
    p = scenarios.plume_batch(1, 3, sizes=(32,), iters=20)[0]
    g = Simulation(p)
    g.add_velocity_noise(3, 0.5)
    g.step(2)
    g.sync()
    o = OracleSim(p, precision="double")
    o.set_topology(g.get_topology())
    for f in ["density", "temperature", "vapor", "vel_x", "vel_y", "vel_z", "fluidity"]:
        o.set_field(f, g.get_field(f).astype(np.float64))
    nq, nc = p.n_scalars, 64 * p.max_blocks
    alloc = np.repeat(o.get_topology()["pos"][:, 3] >= 0, 64)
    rng = np.random.default_rng(9)
    lam = (rng.standard_normal((3 + nq) * nc) * np.tile(alloc, 3 + nq)).astype(np.float32)
    li = torch.from_numpy(lam).cuda()
    lo = torch.empty_like(li)
    g.adjoint_step_full(li, lo)
    torch.cuda.synchronize()
    mv, rf = g.get_last_adapt()
    assert len(mv) + len(rf) > 0
    jo = o.adjoint_step_full(lam.astype(np.float64), moves=mv, refines=rf)
    jg = lo.cpu().numpy().astype(np.float64)
    for k, name in enumerate(["v_x", "v_y", "v_z", "density", "temperature", "vapor"]):
        a, b = jg[k * nc:(k + 1) * nc], jo[k * nc:(k + 1) * nc]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        print(f"{name}: GPU vs FP64 host adjoint, relative L2 {rel:.2e}")
        assert rel <= 1e-3, (name, rel)


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
        the dense density. Backward: the full adjoint of each step in reverse,
        the state before each step recomputed from the checkpoint taken every
        EVERY steps."""

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
            nc = 64 * sim.params.max_blocks
            nplanes = 3 + sim.params.n_scalars
            lam = torch.zeros(nplanes * nc, device="cuda")
            sim.adjoint_dense(g_rho.contiguous(), lam[3 * nc:4 * nc])  # sim holds the final state
            lam_e = torch.zeros(EM_N ** 3, device="cuda")
            nxt = torch.empty_like(lam)
            for t in range(STEPS, 0, -1):
                seg = (t - 1) // EVERY * EVERY
                sim.load_state(ckpt[seg])
                if t - 1 > seg:
                    sim.step(t - 1 - seg)
                sim.adjoint_step_full(lam, nxt, lam_e)  # steps t-1 -> t itself
                lam, nxt = nxt, lam
            torch.cuda.synchronize()
            return lam_e, None, None

    return Rollout


@pytest.fixture(scope="module")
def buoyant4():
    import torch
    from dcgrid_gb300 import Simulation
    p = buoyant()
    s = Simulation(p)
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


def test_buoyant_rollout_gradient_matches_central_differences(buoyant4):
    import torch
    g, E0, loss_of = buoyant4["grad"], buoyant4["E0"].detach(), buoyant4["loss_of"]
    s = buoyant4["sim"]
    st = s.stats()
    assert st.device_error == 0
    eps = 1e-3
    rng = np.random.default_rng(8)
    errs = []
    for _ in range(8):
        d = torch.from_numpy(rng.standard_normal(EM_N ** 3).astype(np.float32)).cuda()
        d = d / d.norm()
        with torch.no_grad():
            fd = (loss_of(E0 + eps * d) - loss_of(E0 - eps * d)).item() / (2 * eps)
        an = float((g * d.double()).sum())
        errs.append(abs(fd - an) / max(abs(fd), 1e-30))
    print("buoyant rollout, central-difference relative errors:", [f"{e:.2e}" for e in errs])
    assert max(errs) <= 1e-2, errs


def test_buoyant_rollout_gradient_matches_fp64_host_adjoint(buoyant4):
    import os
    from oracle.pyoracle import OracleSim, set_threads
    set_threads(os.cpu_count() or 1)
    p, s = buoyant4["p"], buoyant4["sim"]
    E0 = buoyant4["E0"].detach().cpu().numpy().astype(np.float64)
    target = buoyant4["target"].cpu().numpy().astype(np.float64)
    # the GPU run's adaptation decisions, step by step (stage calls)
    s.load_state(buoyant4["state0"])
    s.set_emission(buoyant4["E0"].detach().contiguous())
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
    nc = 64 * p.max_blocks
    lam = np.zeros((3 + p.n_scalars) * nc)
    lam_rho = np.zeros(nc)
    o.adjoint_dense(2.0 * (rho - target), lam_rho)
    lam[3 * nc:4 * nc] = lam_rho
    lam_e = np.zeros(EM_N ** 3)
    for t in range(STEPS, 0, -1):
        seg = (t - 1) // EVERY * EVERY
        o.copy_state_from(ckpt[seg])
        for k in range(seg, t - 1):
            step(o, k)
        mv, rf = decisions[t - 1]
        lam = o.adjoint_step_full(lam, lam_e, moves=mv, refines=rf)
    g = buoyant4["grad"].cpu().numpy()
    rel = np.linalg.norm(g - lam_e) / np.linalg.norm(lam_e)
    print("buoyant rollout: GPU FP32 vs FP64 host adjoint gradient, relative L2:", f"{rel:.2e}")
    assert rel <= 1e-3, rel


def test_full_adjoint_refuses_what_it_does_not_transpose():
    import torch
    from dcgrid_gb300 import DcgError, Simulation
    p = buoyant(32, 2, iters=10, em_n=8)
    p.precision = capi.PRECISION_MIXED_FP16
    s = Simulation(p)
    n = (3 + p.n_scalars) * 64 * p.max_blocks
    a, b = torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
    with pytest.raises(DcgError):
        s.adjoint_step_full(a, b)
    q = buoyant(32, 2, iters=10, em_n=8)
    q.defect_passes = 1
    with pytest.raises(DcgError):
        Simulation(q).adjoint_step_full(a, b)
