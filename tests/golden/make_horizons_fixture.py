"""Writes horizons_synthetic.txt: a synthetic vector table in the layout of NASA JPL Horizons
text output (a free-text header, "$$SOE", records of a date line, an X / Y / Z line, a
VX / VY / VZ line and an LT / RG / RR line, "$$EOE", a footer). The numbers are seeded random
values, not ephemerides. A few records are broken on purpose to exercise the parser's record
boundaries: a date line without a position line after it, a position line without a velocity
line, a date text that is not a number, and values glued to their '=' (the layout the
reference's token rule reads). Run:  python tests/golden/make_horizons_fixture.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "horizons_synthetic.txt")


def e(v):
    """Horizons-style scientific notation: a sign column, 15 mantissa digits."""
    s = f"{v:.15E}"
    return s if v < 0 else " " + s


def main():
    rng = np.random.default_rng(2024)
    lines = [
        "Synthetic vector table for parser tests (values are random, not an ephemeris)",
        "Target body name: Test body (000)",
        "Output units    : KM-S",
        "2451545.0 = a header line that starts with a number",
        "*******************************************************************************",
        "$$SOE",
    ]
    jd = 2460000.5
    for r in range(24):
        x = rng.normal(0, 1e8, 3)
        v = rng.normal(0, 20, 3)
        date = f"{jd + r:.9f} = A.D. 2023-Feb-{(r % 28) + 1:02d} 00:00:00.0000 TDB "
        if r == 5:  # not a number before the '='
            date = "24600x5.5 = A.D. 2023-Feb-06 00:00:00.0000 TDB "
        lines.append(date)
        if r == 8:  # a date line followed by another date line: no record
            continue
        if r == 11:  # values glued to their labels
            lines.append(f" X={x[0]:.15E} Y={x[1]:.15E} Z={x[2]:.15E}")
        else:
            lines.append(f" X ={e(x[0])} Y ={e(x[1])} Z ={e(x[2])}")
        if r == 14:  # a position line without a velocity line: no record
            lines.append(f" LT={e(abs(x[0]) / 3e5)} RG={e(abs(x[1]))} RR={e(v[0])}")
            continue
        if r == 17:
            lines.append(f" VX={v[0]:.15E} VY={v[1]:.15E} VZ={v[2]:.15E}")
        else:
            lines.append(f" VX={e(v[0])} VY={e(v[1])} VZ={e(v[2])}")
        lines.append(f" LT={e(abs(x[0]) / 3e5)} RG={e(abs(x[1]))} RR={e(v[0])}")
    lines += [
        "$$EOE",
        "*******************************************************************************",
        "Footer text; $$SOE and $$EOE mark the data region.",
    ]
    with open(OUT, "w") as f:
        f.write("\n".join(lines) + "\n")
    print(OUT)


if __name__ == "__main__":
    main()
