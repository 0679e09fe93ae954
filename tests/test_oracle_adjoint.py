"""The differentiable-trajectory oracles against each other (CPU only).

The FP64 direct-sum adjoint must match central differences of the frozen-list map at theta = 0,
where every node is opened and the frozen lists are exactly all pairs; at theta = 0.5 the
frozen-list map must replay its own recorded trajectory exactly and use fewer entries."""
import numpy as np

from oracle.oracle import FrozenTrajectory, direct_adjoint


def system(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.normal(size=(n, 3))
    vel = rng.normal(size=(n, 3)) * 0.3
    mass = rng.uniform(0.5, 1.5, n) / n
    return pos, vel, mass


def test_direct_adjoint_matches_frozen_theta0_differences(orc):
    n, nsteps, dt, eps = 96, 12, 1e-2, 0.05
    pos, vel, mass = system(n, 0)
    fr = FrozenTrajectory(orc, pos, vel, mass, dt, 0.0, eps, 1.0, 1, nsteps, nthreads=2)
    assert fr.entries() == n * (n - 1) * (nsteps + 1)
    target = pos + 0.1
    xo, _ = fr.run(pos, vel, mass)
    dl = 2.0 * (xo - target) / n
    xd, _, gx, gv, gm = direct_adjoint(orc, pos, vel, mass, dt, eps, nsteps, dl, nthreads=2)
    assert np.abs(xd - xo).max() < 1e-13

    def loss(x, v, m):
        return float(np.mean(np.sum((fr.run(x, v, m)[0] - target) ** 2, axis=1)))

    rng = np.random.default_rng(1)
    h = 1e-6
    for _ in range(8):
        i, a = int(rng.integers(n)), int(rng.integers(3))
        for arr, g, k in ((pos, gx, 0), (vel, gv, 1)):
            p, m_ = arr.copy(), arr.copy()
            p[i, a] += h
            m_[i, a] -= h
            args_p = [pos, vel, mass]
            args_m = [pos, vel, mass]
            args_p[k], args_m[k] = p, m_
            fd = (loss(*args_p) - loss(*args_m)) / (2 * h)
            assert abs(fd - g[i, a]) <= 1e-6 * abs(fd) + 1e-10
        hm = 1e-4 * mass[i]  # relative step: masses are ~1/n
        mp, mm = mass.copy(), mass.copy()
        mp[i] += hm
        mm[i] -= hm
        fd = (loss(pos, vel, mp) - loss(pos, vel, mm)) / (2 * hm)
        assert abs(fd - gm[i]) <= 1e-6 * abs(fd) + 1e-10


def test_frozen_replay_is_deterministic(orc):
    n, nsteps = 300, 6
    pos, vel, mass = system(n, 2)
    fr = FrozenTrajectory(orc, pos, vel, mass, 1e-2, 0.5, 0.05, 1.0, 4, nsteps, nthreads=2)
    assert 0 < fr.entries() < n * (n - 1) * (nsteps + 1)
    xo, vo = fr.run(pos, vel, mass)
    assert np.array_equal(xo, fr.final_pos) and np.array_equal(vo, fr.final_vel)
