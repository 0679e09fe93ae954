"""Generates the scene and ephemeris golden fixtures from REF-LITERAL's scene library.

oracle/_ref/libbhref_solar.so is the reference's own SetupSolarSystem (src/PhysicsHelpers.hpp)
and parseHorizonsFilez (src/SolarSystem.c), compiled unmodified by oracle/build_oracle.py. It
can only be built where the reference checkout exists, so its outputs are frozen here:

    ref_scene.npz     SetupSolarSystem with the library's counter-based draws (seed 7) for
                      n = 1, 9, 10, 15, 64 and 4444 (the app's own body count): rows
                      x, y, z, vx, vy, vz, m (FP64, SI units)
    ref_horizons.npz  parseHorizonsFilez on horizons_synthetic.txt (written by
                      make_horizons_fixture.py): rows julianDate, X, Y, Z, VX, VY, VZ

Run:  python tests/golden/make_scene_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402
from oracle.oracle import RefScene  # noqa: E402

SEED = 7
SIZES = (1, 9, 10, 15, 64, 4444)


def main():
    if build_oracle.build_ref_solar() is None:
        raise SystemExit("reference checkout not available")
    ref = RefScene()
    scene = {f"n{n}": ref.solar_system(SEED, n) for n in SIZES}
    np.savez_compressed(os.path.join(HERE, "ref_scene.npz"), seed=np.array([SEED]), **scene)
    rec = ref.parse_horizons(os.path.join(HERE, "horizons_synthetic.txt"))
    np.savez_compressed(os.path.join(HERE, "ref_horizons.npz"), records=rec)
    for f in ("ref_scene.npz", "ref_horizons.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
