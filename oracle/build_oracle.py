"""Builds the oracle libraries (test infrastructure only).

    oracle/_build/liboracle.so  the CPU restatement (oracle/bh_oracle.cpp); built everywhere.
    oracle/_ref/libbhref.so     REF-LITERAL: the reference's own hot-path translation units
                                src/{MathUtils,Body,OctantUtils,HashedNode,HashedOctree}.cpp,
                                compiled unmodified from the reference checkout (read in place,
                                never copied) against oracle/ref_shim/ofMain.h, plus the C-ABI
                                harness oracle/ref_harness.cpp. Built only where the reference
                                checkout exists (REFERENCE_ROOT, the checkout's root).

Both use g++ -O2 -ffp-contract=off without -march flags, so no FMA contraction changes the
FP64 results.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout (read in place; this recipe and reference_path() are the only places
# that name it): REFERENCE_ROOT overrides the container's mount point
REFERENCE_ROOT = os.environ.get("REFERENCE_ROOT", "/root/reference")
REF_SRC = os.environ.get("REFERENCE_SRC", os.path.join(REFERENCE_ROOT, "src"))


def reference_path(*parts):
    """A path inside the reference checkout, or None where the checkout is absent (the GPU
    host, any other machine)."""
    p = os.path.join(REFERENCE_ROOT, *parts)
    return p if os.path.exists(p) else None
REF_TUS = ["MathUtils.cpp", "Body.cpp", "OctantUtils.cpp", "HashedNode.cpp", "HashedOctree.cpp"]
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread"]


def build_restatement():
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle.so")
    subprocess.run(["g++", *FLAGS, "-o", out + ".tmp", os.path.join(HERE, "bh_oracle.cpp")], check=True)
    os.replace(out + ".tmp", out)
    return out


def build_ref():
    """Returns the library path, or None when the reference checkout is absent."""
    if not all(os.path.exists(os.path.join(REF_SRC, f)) for f in REF_TUS):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libbhref.so")
    cmd = ["g++", *FLAGS, "-w", "-I" + os.path.join(HERE, "ref_shim"), "-I" + REF_SRC, "-o", out + ".tmp",
           os.path.join(HERE, "ref_harness.cpp")] + [os.path.join(REF_SRC, f) for f in REF_TUS]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


SOLAR_CXX = ["MathUtils.cpp", "Body.cpp"]
SOLAR_C = ["SolarSystem.c", "StringUtilities.c", "FileUtilities.c", "DataExtraction.c", "GeneralUtilities.c",
           "CommonDefinitions.c"]


def build_ref_solar():
    """REF-LITERAL for the app's scene set-up and ephemeris ingest: the reference's
    SetupSolarSystem (src/PhysicsHelpers.hpp) and parseHorizonsFilez (src/SolarSystem.c) with
    their C utilities, compiled unmodified against the shim, plus oracle/ref_solar_harness.cpp.
    Returns the library path, or None when the reference checkout is absent."""
    if not all(os.path.exists(os.path.join(REF_SRC, f)) for f in SOLAR_CXX + SOLAR_C + ["PhysicsHelpers.hpp"]):
        return None
    out_dir = os.path.join(HERE, "_ref")
    obj_dir = os.path.join(out_dir, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    objs = []
    for f in SOLAR_C:
        obj = os.path.join(obj_dir, f[:-2] + ".o")
        pre = ["-include", os.path.join(HERE, "ref_shim", "isnan_int.h")] if f == "GeneralUtilities.c" else []
        subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-w", *pre, "-I" + REF_SRC, "-c",
                        os.path.join(REF_SRC, f), "-o", obj], check=True)
        objs.append(obj)
    out = os.path.join(out_dir, "libbhref_solar.so")
    cmd = ["g++", *FLAGS, "-w", "-I" + os.path.join(HERE, "ref_shim"), "-I" + REF_SRC, "-o", out + ".tmp",
           os.path.join(HERE, "ref_solar_harness.cpp")] + [os.path.join(REF_SRC, f) for f in SOLAR_CXX] + objs
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build_all():
    return build_restatement(), build_ref(), build_ref_solar()


if __name__ == "__main__":
    print(build_all())
