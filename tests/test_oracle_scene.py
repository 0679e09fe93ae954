"""The reference app's scene set-up and ephemeris ingest, on the CPU.

  * the oracle's scene restatement against the reference's own SetupSolarSystem (golden vectors
    from REF-LITERAL, and live where the reference checkout exists): bit-exact in FP64;
  * bh_parse_horizons (host code of the library) in literal mode against the reference's own
    parseHorizonsFilez: bit-exact on the synthetic fixture (golden) and on the reference's
    Horizons files (live); in the default mode against an independent parse of the same lines;
  * the parser's error cases.
"""
import os
import re

import numpy as np
import pytest

from conftest import golden
from oracle import oracle as oracle_mod

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "horizons_synthetic.txt")
from oracle.build_oracle import reference_path  # noqa: E402

REF_HORIZONS = reference_path("horizon_results")  # None without the reference checkout


@pytest.fixture(scope="module")
def ref_scene():
    from oracle import build_oracle

    if not os.path.exists(oracle_mod.REF_SCENE_LIB) and build_oracle.build_ref_solar() is None:
        pytest.skip("reference checkout not available: REF-LITERAL scene library cannot be built here")
    return oracle_mod.RefScene()


def test_scene_restatement_matches_golden(orc):
    d = golden("ref_scene.npz")
    seed = int(d["seed"][0])
    for key in d.files:
        if key == "seed":
            continue
        n = int(key[1:])
        assert np.array_equal(orc.solar_system(seed, n), d[key]), key


@pytest.mark.parametrize("seed,n", [(0, 11), (3, 20), (11, 500), (12, 2048)])
def test_scene_restatement_matches_reference_live(orc, ref_scene, seed, n):
    assert np.array_equal(orc.solar_system(seed, n), ref_scene.solar_system(seed, n))


def test_scene_layout(orc):
    s = orc.solar_system(1, 4444)
    assert s[0, 6] == 1.989e30 and not s[0, :6].any()
    r_au = np.linalg.norm(s[:, :3], axis=1) / 149597870700.0
    belt, cloud = s[10:2222], s[2222:]
    assert np.all((belt[:, 6] >= 1e15) & (belt[:, 6] <= 1e21))
    assert np.all((cloud[:, 6] >= 1e12) & (cloud[:, 6] <= 1e17))
    assert np.all((r_au[10:2222] > 2.2 * 0.8) & (r_au[10:2222] < 3.2 * 1.2))
    assert np.median(r_au[2222:]) > 500


def regex_parse(path):
    """Independent parse: the records the reference's scan delimits, each value read as the
    number after its label's '='."""
    lines = open(path).read().split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    start = next(i for i, l in enumerate(lines) if "$$SOE" in l) + 1
    end = next(i for i in range(start, len(lines)) if "$$EOE" in lines[i])
    num = r"\s*=\s*([-+]?[0-9.]+(?:[eE][-+]?[0-9]+)?)"

    def vals(line, labels):
        return [float(re.search(r"(?:^|[ \t])" + lab + num, line).group(1)) for lab in labels]

    out, i = [], start
    while i < end:
        if " = A.D." not in lines[i]:
            i += 1
            continue
        jd_text = lines[i][: lines[i].index("=")]
        try:
            jd = float(jd_text)
        except ValueError:
            jd = 0.0
        i += 1
        if i >= end:
            break
        xl = lines[i]
        i += 1
        if not all(re.search(lab + r" ?=", xl) for lab in ("X", "Y", "Z")):
            continue
        if i >= end:
            break
        vl = lines[i]
        i += 1
        if not all(re.search(lab + r" ?=", vl) for lab in ("VX", "VY", "VZ")):
            continue
        out.append([jd] + vals(xl, ("X", "Y", "Z")) + vals(vl, ("VX", "VY", "VZ")))
    return np.array(out)


def rows(recs):
    return np.column_stack([recs["jd_tdb"], recs["pos"], recs["vel"]])


def test_parse_horizons_literal_matches_golden(bh):
    assert np.array_equal(rows(bh.parse_horizons(FIXTURE, literal=True)), golden("ref_horizons.npz")["records"])


def test_parse_horizons_reads_values(bh):
    got = rows(bh.parse_horizons(FIXTURE))
    want = regex_parse(FIXTURE)
    assert got.shape == want.shape == golden("ref_horizons.npz")["records"].shape
    assert np.array_equal(got, want)
    # the literal rule drops every value whose '=' is not glued to the number
    lit = rows(bh.parse_horizons(FIXTURE, literal=True))
    assert np.array_equal(lit[:, 0], got[:, 0])
    assert (lit[:, 1:4] == 0).mean() > 0.9 and (got[:, 1:4] != 0).all()


@pytest.mark.skipif(REF_HORIZONS is None, reason="reference checkout not available")
def test_parse_horizons_reference_files(bh, ref_scene):
    files = sorted(f for f in os.listdir(REF_HORIZONS) if f.startswith("horizons_results_") and f.endswith(".txt"))
    assert files
    for f in files:
        path = os.path.join(REF_HORIZONS, f)
        assert np.array_equal(rows(bh.parse_horizons(path, literal=True)), ref_scene.parse_horizons(path)), f
        assert np.array_equal(rows(bh.parse_horizons(path)), regex_parse(path)), f


def test_parse_horizons_errors_and_counting(bh, tmp_path):
    lib = bh.load()
    import ctypes

    cnt = ctypes.c_size_t(99)
    assert lib.bh_parse_horizons(str(tmp_path / "missing.txt").encode(), 0, None, 0, ctypes.byref(cnt)) == 1
    empty = tmp_path / "no_region.txt"
    empty.write_text("2460000.5 = A.D. 2023 TDB\n X = 1 Y = 2 Z = 3\n VX= 1 VY= 2 VZ= 3\n")
    assert lib.bh_parse_horizons(str(empty).encode(), 0, None, 0, ctypes.byref(cnt)) == 9
    assert lib.bh_parse_horizons(FIXTURE.encode(), 2, None, 0, ctypes.byref(cnt)) == 1
    assert lib.bh_parse_horizons(FIXTURE.encode(), 0, None, 0, None) == 1
    # count only, then a short buffer: the count is the full count, the first records written
    assert lib.bh_parse_horizons(FIXTURE.encode(), 0, None, 0, ctypes.byref(cnt)) == 0
    full = bh.parse_horizons(FIXTURE)
    assert cnt.value == len(full)
    part = np.zeros(3, bh.EPHEMERIS_DTYPE)
    assert lib.bh_parse_horizons(FIXTURE.encode(), 0, part.ctypes.data, 3, ctypes.byref(cnt)) == 0
    assert cnt.value == len(full) and np.array_equal(rows(part), rows(full[:3]))
    # a final line without a newline still counts; an empty region gives zero records
    tail = tmp_path / "tail.txt"
    tail.write_text("$$SOE\n2460000.5 = A.D. 2023 TDB\n X =-1.5E+02 Y = 2 Z = 3\n VX= 1 VY=-2 VZ= 3\n$$EOE")
    got = rows(bh.parse_horizons(str(tail)))
    assert np.array_equal(got, [[2460000.5, -150.0, 2.0, 3.0, 1.0, -2.0, 3.0]])
    lit = rows(bh.parse_horizons(str(tail), literal=True))
    assert np.array_equal(lit, [[2460000.5, 0.0, 0.0, 0.0, 0.0, -2.0, 0.0]])
    none = tmp_path / "none.txt"
    none.write_text("$$SOE\n$$EOE\n")
    assert lib.bh_parse_horizons(str(none).encode(), 0, None, 0, ctypes.byref(cnt)) == 9


def test_bodies_from_ephemerides(bh):
    t = bh.parse_horizons(FIXTURE)
    pm, vel = bh.bodies_from_ephemerides([t, t], [1.0, 2.0], record=2)
    assert np.allclose(pm[0, :3], t["pos"][2] * 1e3) and pm[1, 3] == 2.0
    assert np.allclose(vel[1, :3], t["vel"][2] * 1e3)
