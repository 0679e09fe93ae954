"""Batched ensembles: one bh_batch_step over many systems against the plain path per system.

Each system of the ensemble must evolve exactly as it does alone through bh_step: same
permutation (the system's own Morton order inside its body range), and positions, velocities
and accelerations equal up to FP32 rounding (the only difference is the summation order of the
system's FP64 bounds centre)."""
import numpy as np
import pytest

from oracle.oracle import relerr

pytestmark = pytest.mark.gpu


def ensemble(bh, nsys, seed, nmin=40, nmax=3000):
    rng = np.random.default_rng(seed)
    sizes = np.round(np.exp(rng.uniform(np.log(nmin), np.log(nmax), nsys))).astype(int)
    pos, vel = [], []
    for s, n in enumerate(sizes):
        p, v = bh.plummer(seed * 1000 + s, int(n))
        v[:, 3] = np.arange(n, dtype=np.float32)  # body id rides in the unused velocity lane
        pos.append(p)
        vel.append(v)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    return np.concatenate(pos), np.concatenate(vel), off


@pytest.mark.parametrize("leaf,mode", [(8, 1), (1, 0)])
def test_batch_step_matches_plain_per_system(bh, leaf, mode):
    pm, vel, off = ensemble(bh, 37, 5)
    prm = bh.default_params(theta=0.6, eps=0.01, dt=1e-3, leaf_capacity=leaf, multipole=mode, edge_factor=2.0)
    nsteps = 3
    with bh.Simulation(len(pm)) as sim:
        sim.batch_set(pm, vel, off)
        st = sim.batch_step(prm, nsteps)
        assert st.steps == nsteps and st.error_flags == 0
        bp, bv, ba = sim.get_bodies()
    worst = 0.0
    with bh.Simulation(int(np.diff(off).max())) as one:
        for s in range(len(off) - 1):
            a, b = off[s], off[s + 1]
            one.set_bodies(pm[a:b], vel[a:b])
            one.step(prm, nsteps)
            p, v, acc = one.get_bodies()
            assert np.array_equal(bv[a:b, 3], v[:, 3]), f"system {s}: permutation differs"
            assert np.allclose(bp[a:b, :3], p[:, :3], rtol=0, atol=1e-6)
            assert np.allclose(bv[a:b, :3], v[:, :3], rtol=0, atol=1e-6)
            worst = max(worst, float(relerr(ba[a:b], acc).max()))
    assert worst <= 1e-5


def test_batch_then_plain_reuse(bh):
    """A context switches between an ensemble and a single system without stale state."""
    pm, vel, off = ensemble(bh, 5, 9, 100, 400)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=4)
    with bh.Simulation(len(pm)) as sim:
        sim.batch_set(pm, vel, off)
        sim.batch_step(prm, 2)
        sim.set_bodies(pm[: off[1]], vel[: off[1]])
        st = sim.step(prm, 1)
        assert st.error_flags == 0
        sim.batch_set(pm, vel, off)
        st = sim.batch_step(prm, 1)
        assert st.steps == 1


def test_batch_set_rejects_bad_offsets(bh):
    pm, vel = bh.plummer(1, 100)
    with bh.Simulation(100) as sim:
        for off in ([0, 50, 50, 100], [1, 100], [0, 60, 40, 100]):
            with pytest.raises(bh.BHError):
                sim.batch_set(pm, vel, np.array(off, np.uint32))


def test_batch_step_host_matches_batch_step(bh):
    """bh_batch_step_host (host copies beside the batched step) follows bh_batch_step's
    trajectory bit for bit, with page-locked buffers (velocities stored by the walk's kick into
    the mapped output), with the same arrays as input and output, with a velocity output off a
    16-byte boundary (downloaded after the walk), with pageable buffers, and after a plain step
    on the same context (its step graphs must not be reused for the ensemble)."""
    pm, vel, off = ensemble(bh, 23, 3, 50, 2000)
    n = len(pm)
    prm = bh.default_params(theta=0.6, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)
    steps = 4
    ref = []
    with bh.Simulation(n) as a:
        a.batch_set(pm, vel, off)
        for _ in range(steps):
            a.batch_step(prm, 1)
            p, v, _ = a.get_bodies()
            ref.append((p.copy(), v.copy()))
    bufs = [bh.PinnedArray((n, 4)) for _ in range(4)]
    spare = bh.PinnedArray((n + 1, 4))
    unaligned_vo = spare.array.reshape(-1)[1:1 + 4 * n].reshape(n, 4)
    try:
        for mode in ("pinned", "inplace", "unaligned", "pageable", "after_plain"):
            with bh.Simulation(n) as b:
                if mode == "after_plain":
                    b.set_bodies(pm, vel)
                    b.step_host(prm, bufs[0].array, bufs[1].array, bufs[2].array, bufs[3].array)
                b.batch_set(pm, vel, off)
                p, v = pm.copy(), vel.copy()
                for k in range(steps):
                    if mode == "pageable":
                        po, vo = np.zeros_like(p), np.zeros_like(v)
                        b.batch_step_host(prm, p, v, po, vo)
                        p, v = po, vo
                    else:
                        pi, vi, po, vo = (x.array for x in bufs)
                        if mode == "unaligned":
                            vo = unaligned_vo
                        if mode == "inplace":
                            po, vo = pi, vi
                        pi[:] = p
                        vi[:] = v
                        b.batch_step_host(prm, pi, vi, po, vo)
                        p, v = po.copy(), vo.copy()
                    assert np.array_equal(p, ref[k][0]) and np.array_equal(v, ref[k][1]), (mode, k)
    finally:
        for x in bufs:
            x.free()
        unaligned_vo = None
        spare.free()


def test_batch_at_the_system_limit(bh):
    """65 535 systems (the most the 16-bit system ids allow) of 1 to 4 bodies: the ensemble steps,
    sampled systems match their own plain steps, and one more system is refused."""
    rng = np.random.default_rng(11)
    nsys = 65535
    sizes = rng.integers(1, 5, nsys)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    n = int(off[-1])
    pm = np.zeros((n, 4), np.float32)
    pm[:, :3] = rng.normal(0, 1, (n, 3)).astype(np.float32)
    pm[:, 3] = 0.25
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.normal(0, 0.1, (n, 3)).astype(np.float32)
    vel[:, 3] = np.arange(n, dtype=np.float32)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=1, multipole=1, edge_factor=2.0)
    with bh.Simulation(n + 8) as sim:
        sim.batch_set(pm, vel, off)
        st = sim.batch_step(prm, 2)
        assert st.steps == 2 and st.error_flags == 0
        bp, bv, _ = sim.get_bodies()
        with pytest.raises(bh.BHError):
            sim.batch_set(np.concatenate([pm, pm[:1]]), np.concatenate([vel, vel[:1]]),
                          np.concatenate([off, [n + 1]]).astype(np.uint32))
    with bh.Simulation(8) as one:
        for s in list(rng.choice(nsys, 20, replace=False)) + [nsys - 1]:
            a, b = off[s], off[s + 1]
            one.set_bodies(pm[a:b], vel[a:b])
            one.step(prm, 2)
            p, v, _ = one.get_bodies()
            assert np.array_equal(bv[a:b, 3], v[:, 3])
            assert np.allclose(bp[a:b, :3], p[:, :3], rtol=0, atol=1e-6)


def ensemble_4096_offsets(seed=1000, nsys=4096, nmin=256, nmax=65536):
    """The batched-ensemble configuration's layout: 4096 systems, N_s = round(exp(U ln 256 +
    ln 256)) on [256, 65 536] (about 47 M bodies), the same draw as the ensemble benchmark."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 1.0, nsys)
    sizes = np.round(np.exp(u * np.log(nmax / nmin) + np.log(nmin))).astype(np.int64)
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)


def test_batch_step_at_ensemble_4096_size(bh, orc):
    """The full 4096-system ensemble (theta 0.6, eps 0.01, leaf 8, dt 1e-3, per-system Plummer
    spheres from the device generator). After one batched step, a seeded sample of 40 systems
    (at least 8 above 16 384 bodies, where the plain path sorts and builds with its multi-block
    kernels) matches each system's own bh_step; six of them, three above 16 384 bodies, also
    match the oracle's step (same permutation, state within 1e-6, accelerations within the
    reference-walk bars)."""
    off = ensemble_4096_offsets()
    sizes = np.diff(off).astype(np.int64)
    n = int(off[-1])
    prm = bh.default_params(theta=0.6, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)
    rng = np.random.default_rng(11)
    big = np.flatnonzero(sizes > 16384)
    small = np.flatnonzero(sizes <= 16384)
    pick = np.sort(np.concatenate([rng.choice(big, 10, replace=False), rng.choice(small, 30, replace=False)]))
    with bh.Simulation(n) as sim:
        sim.batch_plummer_device(1000, off)
        pm, vel, _ = sim.get_bodies()
        for s in range(len(sizes)):  # body id within its system rides in the unused velocity lane
            vel[off[s]:off[s + 1], 3] = np.arange(sizes[s], dtype=np.float32)
        sim.batch_set(pm, vel, off)
        st = sim.batch_step(prm, 1)
        assert st.steps == 1 and st.error_flags == 0
        bp, bv, ba = sim.get_bodies()
    worst = 0.0
    with bh.Simulation(int(sizes[pick].max())) as one:
        for s in pick:
            a, b = int(off[s]), int(off[s + 1])
            one.set_bodies(pm[a:b], vel[a:b])
            one.step(prm, 1)
            p, v, acc = one.get_bodies()
            assert np.array_equal(bv[a:b, 3], v[:, 3]), f"system {s} ({b - a} bodies): permutation differs"
            assert np.allclose(bp[a:b, :3], p[:, :3], rtol=0, atol=1e-6)
            assert np.allclose(bv[a:b, :3], v[:, :3], rtol=0, atol=1e-6)
            worst = max(worst, float(relerr(ba[a:b], acc).max()))
    assert worst <= 1e-5
    for s in np.concatenate([pick[np.isin(pick, big)][:3], pick[~np.isin(pick, big)][:3]]):
        a, b = int(off[s]), int(off[s + 1])
        out = orc.steps(pm[a:b, :3], vel[a:b, :3], pm[a:b, 3], np.zeros((b - a, 3)), 1e-3, 0.6, 0.01, 2.0, 8, 1, 1,
                        acc_follows_body=1, nthreads=16)
        assert np.array_equal(bv[a:b, 3].astype(np.int64), out["perm"].astype(np.int64)), s
        assert np.allclose(bp[a:b, :3], out["pos"], rtol=0, atol=1e-6)
        assert np.allclose(bv[a:b, :3], out["vel"], rtol=0, atol=1e-6)
        err = relerr(ba[a:b], out["acc"])
        assert np.median(err) <= 1e-5 and np.percentile(err, 99) <= 1e-4, (s, np.median(err), np.percentile(err, 99))
