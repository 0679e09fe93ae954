"""Reverse mode (bh_adjoint_forward / bh_step_backward) against the FP64 oracles.

Loss: mean squared distance of the final positions to a target snapshot, the target coming
from a forward run with masses perturbed by lognormal(0.1) factors. Checks:
  * theta = 0 (every node opened: the tree force is the direct sum) against the FP64
    direct-sum adjoint, over all gradient entries;
  * theta = 0.5 against FP64 central differences of the frozen-list map (the FP64 trajectory
    with its own interaction lists held fixed), on 64 random coordinates;
  * theta = 0.5 at N = 4096 against the FP64 direct-sum adjoint (tree approximation error);
  * checkpoint spacing, repeated backward calls and the state after a backward pass;
  * a torch.autograd.Function over the ABI (test-only) hands back the same gradients.
Errors are norm-wise: |g - g_ref| / |g_ref| per gradient kind (positions, velocities, masses).

The oracles receive the library's own loss cotangent dL/dx_N = 2 (x_N - target) / N, taken at
the library's final state: the residual x_N - target is ~1e-4 while FP32 and FP64 trajectories
differ by ~1e-6, so cotangents taken at each side's own final state would differ by about 1%
before any adjoint arithmetic. With one cotangent the checks measure the adjoint alone (J^T
applied to the same vector); the finite differences are those of the loss linearised at the
final state, L(x0) = dL/dx_N . x_N(x0).
"""
import os

import numpy as np
import pytest

from oracle.oracle import FrozenTrajectory, direct_adjoint

pytestmark = pytest.mark.gpu


def setup(bh, n, seed=1):
    pm, vel = bh.plummer(seed, n)
    rng = np.random.default_rng(2)
    return pm, vel, rng.lognormal(0.0, 0.1, n).astype(np.float32)


def target_of(bh, pm, vel, mfac, prm, nsteps):
    tpm = pm.copy()
    tpm[:, 3] *= mfac
    with bh.Simulation(len(pm)) as sim:
        sim.set_bodies(tpm, vel)
        sim.adjoint_forward(prm, nsteps, nsteps)
        p, _, _ = sim.get_bodies()
    return p[:, :3].astype(np.float64)


def gpu_grads(bh, pm, vel, prm, nsteps, every, target):
    n = len(pm)
    with bh.Simulation(n) as sim:
        sim.set_bodies(pm, vel)
        st = sim.adjoint_forward(prm, nsteps, every)
        assert st.steps == nsteps
        p, v, _ = sim.get_bodies()
        dl = (2.0 * (p[:, :3] - target) / n).astype(np.float32)
        gx, gv, gm = sim.step_backward(dl, None)
    return p, v, gx[:, :3].astype(np.float64), gv[:, :3].astype(np.float64), gm.astype(np.float64), \
        dl.astype(np.float64)


def nrel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def test_theta0_matches_direct_sum_adjoint(bh, orc):
    n, nsteps, every = 1024, 40, 6
    prm = bh.default_params(theta=0.0, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=1.0)
    pm, vel, mfac = setup(bh, n)
    target = target_of(bh, pm, vel, mfac, prm, nsteps)
    p, v, gx, gv, gm, dl = gpu_grads(bh, pm, vel, prm, nsteps, every, target)
    xo, _, rx, rv, rm = direct_adjoint(orc, pm[:, :3], vel[:, :3], pm[:, 3], 1e-3, 0.01, nsteps, dl)
    assert np.abs(p[:, :3] - xo).max() < 1e-5
    ex, ev, em = nrel(gx, rx), nrel(gv, rv), nrel(gm, rm)
    print(f"theta=0 vs FP64 direct-sum adjoint: pos {ex:.2e} vel {ev:.2e} mass {em:.2e}")
    assert ex < 1e-4 and ev < 1e-4 and em < 1e-4


def test_theta05_matches_frozen_list_finite_differences(bh, orc):
    errs = frozen_fd_check(bh, orc, 2048, 40, 7)
    print("theta=0.5 vs FP64 frozen-list central differences:", {k: f"{v:.2e}" for k, v in errs.items()})
    assert all(e < 1e-4 for e in errs.values()), errs


def frozen_fd_check(bh, orc, n, nsteps, every, ncoord=(32, 16, 16), seed=1, nthreads=None, mass_step=1e-4):
    """Adjoint gradients of the GPU path against FP64 central differences of the frozen-list map
    on ncoord = (positions, velocities, masses) random coordinates: h = 1e-4 for positions and
    velocities, mass_step times the mass for masses. Each difference is taken as
    dL/dx_N . (x_N(+h) - x_N(-h)), position by position, before the sum. Returns the norm-wise
    relative error per kind."""
    dt, eps, theta, leaf = 1e-3, 0.01, 0.5, 8
    prm = bh.default_params(theta=theta, eps=eps, dt=dt, leaf_capacity=leaf, multipole=1, edge_factor=1.0)
    pm, vel, mfac = setup(bh, n, seed)
    target = target_of(bh, pm, vel, mfac, prm, nsteps)
    _, _, gx, gv, gm, dl = gpu_grads(bh, pm, vel, prm, nsteps, every, target)
    x0, v0, m0 = pm[:, :3].astype(np.float64), vel[:, :3].astype(np.float64), pm[:, 3].astype(np.float64)
    fr = FrozenTrajectory(orc, x0, v0, m0, dt, theta, eps, 1.0, leaf, nsteps, nthreads=nthreads or os.cpu_count())

    def dloss(plus, minus):  # the loss linearised at the final state, differenced per position
        xp, _ = fr.run(*plus)
        xm, _ = fr.run(*minus)
        return float(np.sum(dl * (xp - xm)))

    rng = np.random.default_rng(3)
    h = 1e-4
    got = {"pos": [], "vel": [], "mass": []}
    want = {"pos": [], "vel": [], "mass": []}
    for kind, count in zip(("pos", "vel", "mass"), ncoord):
        for _ in range(count):
            i = int(rng.integers(n))
            if kind == "mass":
                hh = mass_step * m0[i]  # masses are ~1/n: the step is relative to the mass
                mp, mm = m0.copy(), m0.copy()
                mp[i] += hh
                mm[i] -= hh
                fd = dloss((x0, v0, mp), (x0, v0, mm)) / (2 * hh)
                g = gm[i]
            else:
                a = int(rng.integers(3))
                base = x0 if kind == "pos" else v0
                bp, bm = base.copy(), base.copy()
                bp[i, a] += h
                bm[i, a] -= h
                if kind == "pos":
                    fd = dloss((bp, v0, m0), (bm, v0, m0)) / (2 * h)
                    g = gx[i, a]
                else:
                    fd = dloss((x0, bp, m0), (x0, bm, m0)) / (2 * h)
                    g = gv[i, a]
            got[kind].append(g)
            want[kind].append(fd)
    return {k: nrel(np.array(got[k]), np.array(want[k])) for k in got}


def test_adjoint_64k_checkpoints_20_matches_frozen_list_finite_differences(bh, orc):
    """The adjoint configuration's size and checkpoint spacing: N = 65 536 (seed 1), theta 0.5,
    eps 0.01, leaf 8, dt 1e-3, checkpoints every 20 steps, 64 coordinates. The horizon is 24
    steps instead of 200 (a 20-step segment and a 4-step one, so the backward pass recomputes
    from two checkpoints): every finite difference re-runs the FP64 frozen-list trajectory on the
    host, 128 of them, and 200 steps would take the oracle about an hour. Mass steps are 1e-2 of
    the mass: at this N one body's mass moves the final positions by ~1e-12, and with a 1e-4 step
    the difference drowns in FP64 rounding of the O(1) positions (steps of 1e-4, 1e-3 and 1e-2 of
    the mass disagree by up to 2e-3 at the smallest; 1e-3 and 1e-2 agree to 1e-5)."""
    errs = frozen_fd_check(bh, orc, 65536, 24, 20, mass_step=1e-2)
    print("N=65536, 24 steps, checkpoints every 20, vs FP64 frozen-list central differences:",
          {k: f"{v:.2e}" for k, v in errs.items()})
    assert all(e < 1e-4 for e in errs.values()), errs


def test_theta05_n4096_close_to_direct_sum_adjoint(bh, orc):
    n, nsteps, every = 4096, 20, 5
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=1.0)
    pm, vel, mfac = setup(bh, n)
    target = target_of(bh, pm, vel, mfac, prm, nsteps)
    _, _, gx, gv, gm, dl = gpu_grads(bh, pm, vel, prm, nsteps, every, target)
    _, _, rx, rv, rm = direct_adjoint(orc, pm[:, :3], vel[:, :3], pm[:, 3], 1e-3, 0.01, nsteps, dl)
    ex, ev, em = nrel(gx, rx), nrel(gv, rv), nrel(gm, rm)
    print(f"theta=0.5 N=4096 vs FP64 direct-sum adjoint: pos {ex:.2e} vel {ev:.2e} mass {em:.2e}")
    # measured 3e-6 / 1e-6 / 1e-3: positions and velocities carry only FP32 rounding, the mass
    # gradient the tree approximation (cells whose members' masses enter through M and Q)
    assert ex < 3e-5 and ev < 3e-5 and em < 5e-3


def test_checkpoint_spacing_and_repeat(bh):
    n, nsteps = 1500, 12
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=1.0)
    pm, vel, mfac = setup(bh, n, seed=4)
    target = target_of(bh, pm, vel, mfac, prm, nsteps)
    ref = None
    for every in (1, 5, 12, 50):
        p, v, gx, gv, gm, _ = gpu_grads(bh, pm, vel, prm, nsteps, every, target)
        if ref is None:
            ref = (p, v, gx, gv, gm)
            continue
        assert np.array_equal(p, ref[0]) and np.array_equal(v, ref[1])
        for a, b in zip((gx, gv, gm), ref[2:]):
            assert nrel(a, b) < 1e-5
    with bh.Simulation(n) as sim:
        sim.set_bodies(pm, vel)
        sim.adjoint_forward(prm, nsteps, 4)
        p1, v1, a1 = sim.get_bodies()
        dl = 2.0 * (p1[:, :3] - target) / n
        g1 = sim.step_backward(dl, None)
        p2, v2, a2 = sim.get_bodies()  # backward leaves the bodies in the final state
        assert np.array_equal(p1, p2) and np.array_equal(v1, v2) and np.array_equal(a1, a2)
        g2 = sim.step_backward(dl, None)
        for a, b in zip(g1, g2):
            assert nrel(a, b) < 1e-5
        # velocity-only loss
        gvv = sim.step_backward(None, np.ones((n, 3), np.float32))
        assert np.isfinite(gvv[0]).all() and np.abs(gvv[1][:, :3]).max() > 0.5


def test_adjoint_rejects_unsupported(bh):
    pm, vel = bh.plummer(7, 256)
    with bh.Simulation(256) as sim:
        sim.set_bodies(pm, vel)
        with pytest.raises(bh.BHError):
            sim.step_backward(np.zeros((256, 3), np.float32), None)  # no forward pass yet
        for kw in (dict(multipole=0), dict(eps=0.0)):
            prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1)
            for k, v in kw.items():
                setattr(prm, k, v)
            with pytest.raises(bh.BHError):
                sim.adjoint_forward(prm, 3, 1)


def test_torch_autograd_function(bh):
    torch = pytest.importorskip("torch")
    from torch_adjoint import trajectory

    n, nsteps, every = 1024, 10, 3
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=1.0)
    pm, vel, mfac = setup(bh, n)
    target = target_of(bh, pm, vel, mfac, prm, nsteps)
    _, _, gx, gv, gm, _ = gpu_grads(bh, pm, vel, prm, nsteps, every, target)
    x0 = torch.tensor(pm[:, :3], requires_grad=True)
    v0 = torch.tensor(vel[:, :3], requires_grad=True)
    m0 = torch.tensor(pm[:, 3], requires_grad=True)
    with bh.Simulation(n) as sim:
        xn, vn = trajectory(x0, v0, m0, sim, prm, nsteps, every)
        loss = ((xn.double() - torch.from_numpy(target)) ** 2).sum(1).mean()
        loss.backward()
    assert nrel(x0.grad.numpy(), gx) < 1e-5
    assert nrel(v0.grad.numpy(), gv) < 1e-5
    assert nrel(m0.grad.numpy(), gm) < 1e-5
