"""Conservation diagnostics (bh_energy_diag) against FP64 references.

  * theta = 0: the tree potential is the direct sum, per body within FP32 rounding of the FP64
    oracle's potential;
  * theta = 0.5 (quadrupole): per-body potential within 1e-3 (median) of the direct sum;
  * kinetic energy, momentum, angular momentum, mass, centre of mass: FP64 sums of the state;
  * a 100-step run of the small Plummer configuration conserves energy and momentum.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def state_moments(p, v):
    m = p[:, 3].astype(np.float64)
    x = p[:, :3].astype(np.float64)
    u = v[:, :3].astype(np.float64)
    return dict(kinetic=0.5 * np.sum(m * np.sum(u * u, 1)), momentum=(m[:, None] * u).sum(0),
                angular=(m[:, None] * np.cross(x, u)).sum(0), mass=m.sum(), com=(m[:, None] * x).sum(0) / m.sum())


@pytest.mark.parametrize("theta,leaf", [(0.0, 1), (0.0, 8), (0.5, 1), (0.5, 8)])
def test_potential_vs_direct_sum(bh, orc, theta, leaf):
    n, eps = 4096, 0.01
    pm, vel = bh.plummer(21, n)
    with bh.Simulation(n) as sim:
        sim.set_bodies(pm, vel)
        c, size = sim.bounds()
        sim.build(c, 2 * size, leaf, bh.BH_MULTIPOLE_QUADRUPOLE)
        e, pot = sim.energy(theta, eps, potential=True)
        p, v, _ = sim.get_bodies()
    pos, mass = p[:, :3].astype(np.float64), p[:, 3].astype(np.float64)
    _, ref = orc.direct(pos, mass, eps, potential=True)
    err = np.abs(pot - ref) / np.abs(ref)
    w_ref = 0.5 * np.sum(mass * ref)
    if theta == 0.0:
        assert np.median(err) < 1e-6 and err.max() < 1e-5
        assert abs(e["potential"] - w_ref) < 1e-6 * abs(w_ref)
    else:
        assert np.median(err) < 1e-3
        assert abs(e["potential"] - w_ref) < 1e-3 * abs(w_ref)
    mom = state_moments(p, v)
    assert abs(e["kinetic"] - mom["kinetic"]) < 1e-10 * mom["kinetic"]
    assert np.allclose(e["momentum"], mom["momentum"], rtol=0, atol=1e-10)
    assert np.allclose(e["angular_momentum"], mom["angular"], rtol=0, atol=1e-10)
    assert abs(e["mass"] - mom["mass"]) < 1e-12 and np.allclose(e["com"], mom["com"], atol=1e-10)
    assert e["total"] == e["kinetic"] + e["potential"]


def test_energy_and_momentum_conservation(bh):
    """The small Plummer configuration (N = 16384, theta 0.5, eps 0.01, leaf 1, dt 1e-3) over
    100 KDK steps with quadrupoles."""
    n = 16384
    pm, vel = bh.plummer(0, n)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=1, multipole=1, edge_factor=2.0,
                            acc_follows_body=1)
    with bh.Simulation(n) as sim:
        sim.set_bodies(pm, vel)
        sim.step(prm, 1)
        e0 = sim.energy(0.5, 0.01)
        sim.step(prm, 100)
        e1 = sim.energy(0.5, 0.01)
        p, v, _ = sim.get_bodies()
    drift = abs(e1["total"] - e0["total"]) / abs(e0["total"])
    scale = np.sum(p[:, 3].astype(np.float64) * np.linalg.norm(v[:, :3].astype(np.float64), axis=1))
    dp = np.linalg.norm(np.array(e1["momentum"]) - np.array(e0["momentum"])) / scale
    print(f"energy drift {drift:.2e}, momentum drift {dp:.2e} over 100 steps")
    assert e0["total"] < 0 and drift < 1e-3 and dp < 1e-4


def test_energy_needs_a_tree(bh):
    pm, vel = bh.plummer(3, 100)
    with bh.Simulation(100) as sim:
        sim.set_bodies(pm, vel)
        with pytest.raises(bh.BHError):
            sim.energy(0.5, 0.01)
