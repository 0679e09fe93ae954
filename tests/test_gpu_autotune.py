"""Walk autotuner (bh_autotune_walk): every launch shape runs the same walk, the chosen one is
kept by the context, and the results stay those of the default shape (same interaction
counts, accelerations within FP32 summation-order differences)."""
import numpy as np
import pytest

from oracle.oracle import relerr

pytestmark = pytest.mark.gpu


def test_autotune_plain_tree(bh):
    n = 200000
    pm, vel = bh.plummer(5, n)
    with bh.Simulation(n) as sim:
        sim.set_bodies(pm, vel)
        with pytest.raises(bh.BHError):
            sim.autotune(0.5, 0.01)  # no tree yet
        c, size = sim.bounds()
        sim.build(c, 2 * size, 8, bh.BH_MULTIPOLE_QUADRUPOLE)
        a0, st0 = sim.force(0.5, 0.01, stats=True)
        r = sim.autotune(0.5, 0.01, trials=2)
        assert len(r["variants"]) >= 5 and 0 <= r["best"] < len(r["variants"])
        assert all(v["ms"] > 0 for v in r["variants"])
        assert r["variants"][r["best"]]["ms"] == min(v["ms"] for v in r["variants"])
        a1, st1 = sim.force(0.5, 0.01, stats=True)
        assert st1.interactions_cell == st0.interactions_cell and st1.interactions_p2p == st0.interactions_p2p
        assert float(relerr(a1, a0).max()) < 1e-5
        with pytest.raises(bh.BHError):
            sim.autotune(0.5, 0.0)  # the tuned walk is the positive-softening one


def test_autotune_batched_then_step(bh):
    rng = np.random.default_rng(4)
    sizes = rng.integers(100, 3000, 40)
    pos, vel = [], []
    for s, k in enumerate(sizes):
        p, v = bh.plummer(77 + s, int(k))
        pos.append(p)
        vel.append(v)
    pm, vv = np.concatenate(pos), np.concatenate(vel)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    prm = bh.default_params(theta=0.6, eps=0.01, dt=1e-3, leaf_capacity=8, multipole=1, edge_factor=2.0)
    out = []
    for tune in (False, True):
        with bh.Simulation(len(pm)) as sim:
            sim.batch_set(pm, vv, off)
            sim.batch_step(prm, 1)
            if tune:
                r = sim.autotune(0.6, 0.01, trials=2)
                assert all(v["ms"] > 0 for v in r["variants"])
            sim.batch_step(prm, 2)
            out.append(sim.get_bodies())
    assert np.allclose(out[0][0], out[1][0], rtol=0, atol=1e-5)
    assert float(np.median(relerr(out[0][2], out[1][2]))) < 1e-5


@pytest.mark.parametrize("variant", range(12))
def test_every_walk_variant_matches_oracle(bh, orc, variant):
    """Each launch shape (cell-evaluation form, group size) the tuner can pick gives the reference's
    interaction sets and accelerations within the parity bars. The body count leaves the last
    group partly empty (lanes outside every mask)."""
    n = 20011
    pm, vel = bh.plummer(9, n)
    with bh.Simulation(n) as sim:
        sim.set_bodies(pm, vel)
        sim.set_walk_variant(variant)
        c, size = sim.bounds()
        sim.build(c, 2 * size, 8, bh.BH_MULTIPOLE_QUADRUPOLE)
        acc, st = sim.force(0.5, 0.01, stats=True)
        p, _, _ = sim.get_bodies()
    pos, mass = p[:, :3].astype(np.float64), p[:, 3].astype(np.float64)
    ref, ncell, npt = orc.force(pos, mass, c, 2 * size, 8, 1, 0.5, 0.01, nthreads=8)
    err = relerr(acc, ref)
    assert float(np.median(err)) <= 1e-5 and float(np.percentile(err, 99)) <= 1e-4
    assert abs(st.interactions_cell - int(ncell.sum())) <= 1e-4 * ncell.sum()


def test_set_walk_variant_rejects_out_of_range(bh):
    with bh.Simulation(10) as sim:
        with pytest.raises(bh.BHError):
            sim.set_walk_variant(99)
