"""The reference app's solar-system scene generated on the device (bh_solar_system_device).

  * against REF-LITERAL's own SetupSolarSystem (golden vectors, same draws): the Sun, planets
    and Moon within FP32 rounding; belt and cloud bodies within 1e-5 except the few whose 100
    Newton steps on Kepler's equation have not converged (eccentricities up to 0.99 from
    E = M), where one ulp of sin / cos moves the end point: at most 0.2 %;
  * the gravitational-unit form is the SI form rescaled;
  * the reference's own (literal) force on its own scene, in SI units: against the oracle's
    literal walk, median <= 1e-5 and p99 <= 1e-4.
"""
import numpy as np
import pytest

from conftest import golden
from oracle.oracle import relerr

pytestmark = pytest.mark.gpu

AU, MSUN, G = 149597870700.0, 1.989e30, 6.67430e-11


def rowerr(got, want):
    """Per-body relative errors of position, velocity and mass."""
    ep = np.linalg.norm(got[:, :3] - want[:, :3], axis=1) / np.maximum(np.linalg.norm(want[:, :3], axis=1), 1e-30)
    ev = np.linalg.norm(got[:, 3:6] - want[:, 3:6], axis=1) / np.maximum(np.linalg.norm(want[:, 3:6], axis=1), 1e-30)
    em = np.abs(got[:, 6] - want[:, 6]) / want[:, 6]
    return np.maximum(np.maximum(ep, ev), em)


def device_scene(sim, seed, n, units=0):
    sim.solar_system_device(seed, n, units)
    p, v, _ = sim.get_bodies()
    return np.column_stack([p[:, :3], v[:, :3], p[:, 3]]).astype(np.float64)


def test_scene_vs_reference_golden(bh):
    d = golden("ref_scene.npz")
    seed = int(d["seed"][0])
    with bh.Simulation(4444) as sim:
        for key in d.files:
            if key == "seed":
                continue
            n = int(key[1:])
            want = d[key].astype(np.float32).astype(np.float64)
            got = device_scene(sim, seed, n)
            err = rowerr(got, want)
            k = min(n, 10)
            assert err[:k].max() <= 2e-7, (key, err[:k])
            if n > 10:
                assert (err[10:] <= 1e-5).mean() >= 0.998, (key, np.sort(err)[-10:])


def test_scene_large_vs_restatement(bh, orc):
    n = 1 << 18
    with bh.Simulation(n) as sim:
        got = device_scene(sim, 3, n)
    want = orc.solar_system(3, n).astype(np.float32).astype(np.float64)
    err = rowerr(got, want)
    assert err[:10].max() <= 2e-7
    assert (err[10:] <= 1e-5).mean() >= 0.998, np.sort(err)[-10:]


def test_scene_gravitational_units(bh):
    n = 5000
    with bh.Simulation(n) as sim:
        si = device_scene(sim, 9, n, 0)
        gu = device_scene(sim, 9, n, 1)
    vu = np.sqrt(G * MSUN / AU)
    scaled = np.column_stack([si[:, :3] / AU, si[:, 3:6] / vu, si[:, 6] / MSUN])
    assert np.allclose(gu, scaled, rtol=2e-6, atol=0)
    with bh.Simulation(4) as sim, pytest.raises(bh.BHError):
        sim.solar_system_device(0, 4, 2)


def test_literal_force_on_scene_si(bh, orc):
    """The reference app's configuration: its own scene, SI units, literal multipoles (the
    pseudo-barycentres the reference walks), theta 0.5, its softening 0.025, leaf capacity 1."""
    n = 4444
    with bh.Simulation(n) as sim:
        sim.solar_system_device(7, n, 0)
        pm, _, _ = sim.get_bodies()
        c, size = sim.bounds()
        sim.morton_keys(size)
        perm = sim.sort_bodies()
        sp = pm[perm]
        edge = 2 * size
        sim.build(c, edge, 1, bh.BH_MULTIPOLE_LITERAL)
        acc = sim.force(0.5, 0.025)
    pos = sp[:, :3].astype(np.float64)
    mass = sp[:, 3].astype(np.float64)
    ref_acc, _, _ = orc.force(pos, mass, c, edge, 1, 0, 0.5, 0.025, nthreads=8)
    err = relerr(acc, ref_acc)
    assert np.median(err) <= 1e-5 and np.percentile(err, 99) <= 1e-4, (np.median(err), np.percentile(err, 99))
    assert np.isfinite(acc).all()
