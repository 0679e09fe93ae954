"""Device initial conditions, snapshot files and node boxes.

  * bh_plummer_device: the Plummer recipe's distribution (enclosed-mass profile against the
    analytic one, isotropy, bound speeds), centre-of-mass frame, masses, virial ratio;
  * bh_batch_plummer_device: every system in its own centre-of-mass frame with its own mass;
  * snapshots: save -> load -> step gives the same state as stepping the original;
  * bh_tree_boxes: node cubes from the reference's child-bounds recurrence.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_plummer_device_distribution(bh):
    n = 200000
    with bh.Simulation(n) as sim:
        sim.plummer_device(3, n, a=1.0, mtot=1.0)
        p, v, acc = sim.get_bodies()
        assert np.all(acc == 0)
        c, size = sim.bounds()
        sim.build(c, 2 * size, 8, bh.BH_MULTIPOLE_QUADRUPOLE)
        e = sim.energy(0.5, 0.01)
    x, u, m = p[:, :3].astype(np.float64), v[:, :3].astype(np.float64), p[:, 3].astype(np.float64)
    assert np.allclose(m, 1.0 / n, rtol=1e-6) and abs(m.sum() - 1.0) < 1e-5
    assert np.abs(x.mean(0)).max() < 1e-6 and np.abs(u.mean(0)).max() < 1e-6
    r = np.linalg.norm(x, axis=1)
    assert r.max() <= 10.05  # r <= 10 before the centre-of-mass shift
    # enclosed mass M(<r) = r^3 / (1 + r^2)^(3/2), renormalised to the r <= 10 truncation
    rs = np.sort(r)
    model = rs ** 3 / (1 + rs ** 2) ** 1.5 / (1000.0 / 101.0 ** 1.5)
    ks = np.abs(np.arange(1, n + 1) / n - model).max()
    assert ks < 5e-3, ks
    # isotropy and bound speeds
    assert np.abs((x / r[:, None]).mean(0)).max() < 1e-2
    vesc = np.sqrt(2.0) * (1 + r ** 2) ** -0.25
    assert np.all(np.linalg.norm(u, axis=1) <= vesc + 5e-3)  # bound before the centre-of-mass shift
    # virial equilibrium 2K / |W| ~ 1 (softened tree potential, finite N)
    q = 2 * e["kinetic"] / abs(e["potential"])
    assert 0.95 < q < 1.05, q


def test_plummer_device_scaling_and_offsets(bh):
    n = 50000
    with bh.Simulation(n) as sim:
        sim.plummer_device(11, n, a=0.1, mtot=0.1, pos_offset=[10, 0, 0], vel_offset=[-0.3, 0.1, 0])
        p, v, _ = sim.get_bodies()
    x, u = p[:, :3].astype(np.float64), v[:, :3].astype(np.float64)
    assert np.allclose(x.mean(0), [10, 0, 0], atol=1e-5) and np.allclose(u.mean(0), [-0.3, 0.1, 0], atol=1e-5)
    assert abs(p[:, 3].astype(np.float64).sum() - 0.1) < 1e-6
    assert np.linalg.norm(x - [10, 0, 0], axis=1).max() <= 1.005


def test_batch_plummer_device(bh):
    rng = np.random.default_rng(5)
    sizes = np.round(np.exp(rng.uniform(np.log(64), np.log(5000), 60))).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    prm = bh.default_params(theta=0.6, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)
    with bh.Simulation(int(off[-1])) as sim:
        sim.batch_plummer_device(1000, off)
        p, v, _ = sim.get_bodies()
        for s in range(len(sizes)):
            a, b = off[s], off[s + 1]
            xs, us, ms = p[a:b, :3].astype(np.float64), v[a:b, :3].astype(np.float64), p[a:b, 3].astype(np.float64)
            assert abs(ms.sum() - 1.0) < 1e-5
            assert np.abs(xs.mean(0)).max() < 1e-6 and np.abs(us.mean(0)).max() < 1e-6
        st = sim.batch_step(prm, 2)
        assert st.steps == 2 and st.error_flags == 0
        # distinct systems get distinct bodies
        assert not np.array_equal(p[off[0]:off[0] + 10], p[off[1]:off[1] + 10])


@pytest.mark.parametrize("ensemble", [False, True])
def test_snapshot_round_trip(bh, tmp_path, ensemble):
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)
    path = str(tmp_path / "state.bhsnap")
    if ensemble:
        off = np.array([0, 500, 1700, 3000], np.uint32)
        n = int(off[-1])
    else:
        n = 5000
    with bh.Simulation(n) as a, bh.Simulation(n) as b:
        if ensemble:
            a.batch_plummer_device(7, off)
            a.batch_step(prm, 3)
        else:
            a.plummer_device(7, n)
            a.step(prm, 3)
        a.save_snapshot(path)
        b.load_snapshot(path)
        for x, y in zip(a.get_bodies(), b.get_bodies()):
            assert np.array_equal(x, y)
        if ensemble:
            a.batch_step(prm, 2)
            b.batch_step(prm, 2)
        else:
            a.step(prm, 2)
            b.step(prm, 2)
        for x, y in zip(a.get_bodies(), b.get_bodies()):
            assert np.array_equal(x, y)
    with open(path, "r+b") as f:
        f.write(b"XXXX")
    with bh.Simulation(n) as c:
        with pytest.raises(bh.BHError):
            c.load_snapshot(path)


def test_tree_boxes(bh):
    n = 20000
    pm, vel = bh.plummer(4, n)
    with bh.Simulation(n) as sim:
        sim.set_bodies(pm, vel)
        c, size = sim.bounds()
        edge = 2 * size
        sim.build(c, edge, 4, bh.BH_MULTIPOLE_QUADRUPOLE)
        t = sim.tree_nodes()
        box, depth, count = sim.tree_boxes()
    assert np.array_equal(count, t["counts"])
    keys = t["keys"].astype(object)
    for i in np.random.default_rng(0).choice(len(keys), 500, replace=False):
        k = int(keys[i])
        d = (k.bit_length() - 1) // 3
        assert depth[i] == d
        cc, s = [float(c[0]), float(c[1]), float(c[2])], float(edge)
        for lvl in range(d - 1, -1, -1):
            o = (k >> (3 * lvl)) & 7
            s = s * 0.5
            for a in range(3):
                cc[a] = cc[a] + ((0.5 if (o >> (2 - a)) & 1 else -0.5) * s)
        assert np.array_equal(box[i], np.array(cc + [s], np.float32))
    # node 0 is the root cube
    assert depth[0] == 0 and box[0, 3] == np.float32(edge)
