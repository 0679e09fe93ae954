"""Edge cases across the entry points: empty states, one or two bodies, ensembles of tiny
systems, and the differentiable path on the smallest inputs."""
import numpy as np
import pytest

from oracle.oracle import direct_adjoint, relerr

pytestmark = pytest.mark.gpu


def test_empty_state(bh, tmp_path):
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1)
    with bh.Simulation(16) as sim:
        sim.set_bodies(np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32))
        st = sim.step(prm, 3)
        assert st.steps == 0
        p, v, a = sim.get_bodies()
        assert p.shape == (0, 4)
        path = str(tmp_path / "empty.bhsnap")
        sim.save_snapshot(path)
        sim.load_snapshot(path)
        assert sim.n == 0


@pytest.mark.parametrize("n", [1, 2])
def test_one_and_two_bodies(bh, n):
    pm = np.array([[0.1, -0.2, 0.3, 0.5], [-0.4, 0.25, 0.0, 0.25]], np.float32)[:n]
    vel = np.zeros((n, 4), np.float32)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=1, multipole=1, edge_factor=2.0)
    with bh.Simulation(4) as sim:
        sim.set_bodies(pm, vel)
        sim.step(prm, 5)
        p, v, acc = sim.get_bodies()
        assert np.all(np.isfinite(p)) and np.all(np.isfinite(acc))
        e = sim.energy(0.5, 0.01)
        box, depth, count = sim.tree_boxes()
        assert count[0] == n and depth[0] == 0
    if n == 1:
        assert np.all(acc[:, :3] == 0) and e["potential"] == 0.0
    else:
        # equal and opposite momenta change: sum m a = 0
        assert np.allclose((p[:, 3:4] * acc[:, :3]).sum(0), 0, atol=1e-6)
        assert e["potential"] < 0


def test_ensemble_of_tiny_systems(bh):
    sizes = [1, 2, 3, 31, 32, 33, 1, 64, 65, 2]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=1, multipole=1, edge_factor=2.0)
    pos, vel = [], []
    for s, k in enumerate(sizes):
        p, v = bh.plummer(500 + s, k)
        v[:, 3] = np.arange(k, dtype=np.float32)
        pos.append(p)
        vel.append(v)
    pm, vv = np.concatenate(pos), np.concatenate(vel)
    with bh.Simulation(len(pm)) as sim:
        sim.batch_set(pm, vv, off)
        sim.batch_step(prm, 3)
        bp, bv, ba = sim.get_bodies()
    with bh.Simulation(max(sizes)) as one:
        for s in range(len(sizes)):
            a, b = off[s], off[s + 1]
            one.set_bodies(pm[a:b], vv[a:b])
            one.step(prm, 3)
            p, v, acc = one.get_bodies()
            assert np.array_equal(bv[a:b, 3], v[:, 3])
            assert np.allclose(bp[a:b], p, rtol=0, atol=1e-6)
            if sizes[s] > 1:
                assert float(relerr(ba[a:b], acc).max()) < 1e-5


def test_adjoint_two_bodies_matches_direct_adjoint(bh, orc):
    pm = np.array([[0.1, -0.2, 0.3, 0.5], [-0.4, 0.25, 0.0, 0.25]], np.float32)
    vel = np.array([[0.0, 0.1, 0.0, 0.0], [0.05, -0.2, 0.0, 0.0]], np.float32)
    prm = bh.default_params(theta=0.5, eps=0.05, dt=1e-2, leaf_capacity=1, multipole=1, edge_factor=2.0)
    dl = np.array([[1.0, -0.5, 0.25], [0.3, 0.2, -0.1]], np.float32)
    with bh.Simulation(2) as sim:
        sim.set_bodies(pm, vel)
        sim.adjoint_forward(prm, 30, 7)
        gx, gv, gm = sim.step_backward(dl, None)
    _, _, rx, rv, rm = direct_adjoint(orc, pm[:, :3], vel[:, :3], pm[:, 3], 1e-2, 0.05, 30, dl.astype(np.float64))
    assert np.allclose(gx[:, :3], rx, rtol=1e-4, atol=1e-6)
    assert np.allclose(gv[:, :3], rv, rtol=1e-4, atol=1e-6)
    assert np.allclose(gm, rm, rtol=1e-4, atol=1e-6)


def test_bounded_wait_times_out_and_context_stays_usable(bh):
    """A device wait on a flag that nothing sets gives up after its limit and reports
    BH_ERR_TIMEOUT; the same context then waits successfully and still steps."""
    lib = bh.load()
    pm, vel = bh.plummer(2, 1000)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1)
    with bh.Simulation(1000) as sim:
        assert lib.bh_check_bounded_wait(sim.h, 0, 20000) == 7  # BH_ERR_TIMEOUT
        assert lib.bh_check_bounded_wait(sim.h, 1, 20000) == 0
        assert lib.bh_check_bounded_wait(sim.h, 0, 0) == 1  # invalid limit
        sim.set_bodies(pm, vel)
        st = sim.step(prm, 2)
        assert st.steps == 2 and st.error_flags == 0


def test_reset_same_count_replays_identically(bh):
    """A new state with the same body count keeps the captured step graphs (re-pairing the
    Morton key buffers); the trajectory must be bit-identical to a fresh context's, also after
    an odd number of steps, a different body count in between, and an ensemble in between."""
    n = 3000
    pm, vel = bh.plummer(5, n)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)

    def run(sim, steps):
        sim.set_bodies(pm, vel)
        sim.step(prm, steps)
        return sim.get_bodies()

    with bh.Simulation(n) as fresh:
        ref3 = run(fresh, 3)
    with bh.Simulation(n) as fresh:
        ref2 = run(fresh, 2)
    with bh.Simulation(n) as sim:
        for steps, ref in [(3, ref3), (3, ref3), (2, ref2), (3, ref3)]:
            got = run(sim, steps)
            for g, r in zip(got, ref):
                assert np.array_equal(g, r)
        pm2, vel2 = bh.plummer(6, n // 2)
        sim.set_bodies(pm2, vel2)
        sim.step(prm, 1)
        got = run(sim, 3)
        for g, r in zip(got, ref3):
            assert np.array_equal(g, r)
        sim.batch_set(np.concatenate([pm[: n // 2], pm2]), np.concatenate([vel[: n // 2], vel2]),
                      [0, n // 2, n])
        sim.batch_step(prm, 2)
        got = run(sim, 3)
        for g, r in zip(got, ref3):
            assert np.array_equal(g, r)


@pytest.mark.parametrize("n,multipole,eps", [(5000, 1, 0.01), (70000, 1, 0.01), (4444, 0, 0.0)])
def test_step_host_matches_step(bh, n, multipole, eps):
    """bh_step_host (upload, step, download; copies overlapped with page-locked buffers) follows
    the same trajectory as bh_step, bit for bit: with page-locked buffers (the walk's kick
    writes the velocities into the mapped output buffer), with the same page-locked arrays as
    input and output (the per-frame pattern), with buffers that change between calls
    (re-capture), with a velocity output 4 bytes off a 16-byte boundary (no direct stores: the
    download follows the walk), with pageable numpy arrays, and with no copies at all; for the
    quadrupole walk and for the literal walk without softening."""
    pm, vel = bh.plummer(8, n)
    prm = bh.default_params(theta=0.5, eps=eps, dt=1e-3, leaf_capacity=8, multipole=multipole, edge_factor=2.0)
    steps = 6
    ref = []
    with bh.Simulation(n) as a:
        a.set_bodies(pm, vel)
        for _ in range(steps):
            a.step(prm, 1)
            p, v, _ = a.get_bodies()
            ref.append((p.copy(), v.copy()))
    bufs = [[bh.PinnedArray((n, 4)) for _ in range(4)] for _ in range(2)]
    spare = bh.PinnedArray((n + 1, 4))
    unaligned_vo = spare.array.reshape(-1)[1:1 + 4 * n].reshape(n, 4)
    try:
        for mode in ("pinned", "inplace", "alternating", "unaligned", "pageable", "none"):
            with bh.Simulation(n) as b:
                b.set_bodies(pm, vel)
                p, v = pm.copy(), vel.copy()
                for k in range(steps):
                    if mode == "none":
                        b.step_host(prm, None, None, None, None)
                        p, v, _ = b.get_bodies()
                    elif mode == "pageable":
                        po, vo = np.zeros_like(p), np.zeros_like(v)
                        b.step_host(prm, p, v, po, vo)
                        p, v = po, vo
                    else:
                        pi, vi, po, vo = (x.array for x in bufs[k % 2 if mode == "alternating" else 0])
                        if mode == "unaligned":
                            vo = unaligned_vo
                        if mode == "inplace":
                            po, vo = pi, vi
                        pi[:] = p
                        vi[:] = v
                        b.step_host(prm, pi, vi, po, vo)
                        p, v = po.copy(), vo.copy()
                    assert np.array_equal(p, ref[k][0]) and np.array_equal(v, ref[k][1]), (mode, k)
    finally:
        for s in bufs:
            for x in s:
                x.free()
        unaligned_vo = None
        spare.free()


def test_caller_stream(bh):
    """bh_set_stream: the context's work runs on a caller's stream (here one made by PyTorch,
    used only as a stream factory) and the trajectory is the same as on the context's own
    stream; NULL returns to the own stream. The stream handle round-trips through
    bh_get_stream."""
    torch = pytest.importorskip("torch")
    import ctypes

    n = 4000
    pm, vel = bh.plummer(11, n)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)
    with bh.Simulation(n) as a:
        a.set_bodies(pm, vel)
        a.step(prm, 4)
        ref = a.get_bodies()
    lib = bh.load()
    user = torch.cuda.Stream()
    with bh.Simulation(n) as b:
        b.set_bodies(pm, vel)
        b.step(prm, 1)  # captures the state-0 graph on the own stream
        assert lib.bh_set_stream(b.h, ctypes.c_void_p(user.cuda_stream)) == 0
        got_stream = ctypes.c_void_p()
        assert lib.bh_get_stream(b.h, ctypes.byref(got_stream), None) == 0
        assert got_stream.value == user.cuda_stream
        b.step(prm, 2)  # one new capture (state 1) while the caller's stream is set
        assert lib.bh_set_stream(b.h, None) == 0
        b.step(prm, 1)
        got = b.get_bodies()
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    # the host-copy step on the caller's stream (its copies still fork to the second stream)
    bufs = [bh.PinnedArray((n, 4)) for _ in range(4)]
    try:
        with bh.Simulation(n) as c:
            c.set_bodies(pm, vel)
            assert lib.bh_set_stream(c.h, ctypes.c_void_p(user.cuda_stream)) == 0
            p, v = pm.copy(), vel.copy()
            for _ in range(4):
                bufs[0].array[:] = p
                bufs[1].array[:] = v
                c.step_host(prm, bufs[0].array, bufs[1].array, bufs[2].array, bufs[3].array)
                p, v = bufs[2].array.copy(), bufs[3].array.copy()
        assert np.array_equal(p, ref[0]) and np.array_equal(v, ref[1])
    finally:
        for x in bufs:
            x.free()


@pytest.mark.parametrize("n", [4444, 70000])
def test_stats_and_no_stats_steps_identical(bh, n):
    """Step graphs record their stage events only for calls that return stats; a context switching
    between the two kinds of call (re-capturing its graphs each time) follows the same trajectory
    bit for bit as one that never asks for stats, for the plain step and the ensemble step."""
    pm, vel = bh.plummer(13, n)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)
    pattern = (True, False, False, True, True, False, True)
    with bh.Simulation(n) as a, bh.Simulation(n) as b:
        a.set_bodies(pm, vel)
        b.set_bodies(pm, vel)
        for want in pattern:
            st = a.step(prm, 1, stats=want)
            b.step(prm, 1, stats=False)
            if want:
                assert st.steps == 1 and st.ms_step > 0 and st.ms_walk > 0
        for x, y in zip(a.get_bodies(), b.get_bodies()):
            assert np.array_equal(x, y)
        off = np.array([0, n // 3, n], np.uint32)
        a.batch_set(pm, vel, off)
        b.batch_set(pm, vel, off)
        for want in pattern[:4]:
            st = a.batch_step(prm, 1, stats=want)
            b.batch_step(prm, 1, stats=False)
            if want:
                assert st.steps == 1 and st.ms_step > 0
        for x, y in zip(a.get_bodies(), b.get_bodies()):
            assert np.array_equal(x, y)
