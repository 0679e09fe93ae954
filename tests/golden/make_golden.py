"""Generates the golden fixtures in this directory from REF-LITERAL.

REF-LITERAL is the reference's own hot-path code (src/{MathUtils,Body,OctantUtils,HashedNode,
HashedOctree}.cpp, unmodified) compiled by oracle/build_oracle.py against a headless ofMain.h.
It can only be built where the reference checkout exists, so its outputs are frozen here as
.npz files; the tests pin the oracle restatement and the GPU path against them anywhere.

Inputs are stored verbatim (FP32 positions), so the fixtures do not depend on the host libm
used by the initial-condition generator. Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402
from oracle import build_oracle  # noqa: E402
from oracle.oracle import RefLiteral  # noqa: E402

THETA = 0.5


def cases(bh):
    rng = np.random.default_rng(12345)
    out = {}
    for n in (1, 2, 3, 33, 100, 1000):
        pm, v = bh.plummer(100 + n, n)
        out[f"plummer_{n}"] = pm
    pm, _ = bh.plummer(7, 512)
    shifted = pm.copy()
    shifted[:, :3] += np.float32(5.0)  # bodies far outside the origin-centred Morton cube
    out["shift_pos"] = shifted
    neg = pm.copy()
    neg[:, :3] -= np.float32(5.0)  # negative scaled coordinates (the wrap path)
    out["shift_neg"] = neg
    disk = pm.copy()
    disk[:, 2] = 0.0  # every z equals the root centre's z: ties of the strict '>'
    out["flat_disk"] = disk
    octant = pm.copy()
    octant[:, :3] = np.abs(octant[:, :3]) + np.float32(0.01)  # all bodies in one octant
    out["one_octant"] = octant
    cube = np.zeros((777, 4), np.float32)
    cube[:, :3] = rng.uniform(-1, 1, (777, 3)).astype(np.float32)
    cube[:, 3] = rng.uniform(0.5, 2.0, 777).astype(np.float32) / 777
    out["uniform_cube"] = cube
    grid = np.zeros((512, 4), np.float32)
    g = np.arange(8, dtype=np.float32) - np.float32(3.5)
    gx, gy, gz = np.meshgrid(g, g, g, indexing="ij")
    grid[:, 0], grid[:, 1], grid[:, 2] = gx.ravel(), gy.ravel(), gz.ravel()
    grid[:, 3] = 1.0 / 512
    out["lattice"] = grid  # positions exactly on power-of-two cell boundaries
    return out


def literal_case(ref, pm):
    pos = pm[:, :3].astype(np.float64)
    mass = pm[:, 3].astype(np.float64)
    c, size = ref.bounds(pos)
    keys = ref.morton_keys(pos, size)
    perm = ref.sort_perm(keys)
    sp, sm = pos[perm], mass[perm]
    rec = dict(pos_m=pm, center=c, size=np.array([size]), keys=keys, perm=perm)
    for tag, ef in (("e1", 1.0), ("e2", 2.0)):
        edge = size * ef
        if size <= 0 or ref.guard(sp, c, edge) != 0:
            rec[f"{tag}_refused"] = np.array([1])
            continue
        t = ref.build(sp, sm, c, edge)
        rec[f"{tag}_node_keys"] = t["keys"]
        rec[f"{tag}_node_counts"] = t["counts"].astype(np.int32)
        rec[f"{tag}_node_mass"] = t["mass"]
        rec[f"{tag}_node_com"] = t["com"]
        rec[f"{tag}_node_child"] = t["child_byte"]
        rec[f"{tag}_node_box"] = t["box"]  # nodeBounds: centre x, y, z and size (FP64)
        acc, ll = ref.force(sp, sm, c, edge, THETA)
        rec[f"{tag}_acc"] = acc
        rec[f"{tag}_list_len"] = ll.astype(np.int32)
    return rec


def main():
    build_oracle.build_all()
    bh = __graft_entry__.package()
    bh.load()
    ref = RefLiteral()
    small = {}
    for name, pm in cases(bh).items():
        for k, v in literal_case(ref, pm).items():
            small[f"{name}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "literal_small.npz"), **small)

    # config 0 size: one Plummer sphere, N = 16384, seed 0 (the app's edge-S geometry)
    pm, vel = bh.plummer(0, 16384)
    rec = literal_case(ref, pm)
    keep = {k: rec[k] for k in ("pos_m", "center", "size", "keys", "perm", "e1_node_keys", "e1_node_counts",
                                "e1_list_len")}
    keep["e1_acc"] = rec["e1_acc"].astype(np.float32)
    keep["e1_node_box"] = rec["e1_node_box"].astype(np.float32)  # as the library returns node boxes
    np.savez_compressed(os.path.join(HERE, "literal_config0.npz"), **keep)

    # three frames of ofApp::update + draw (drawing excluded), app geometry, theta = 0.5
    pm, vel = bh.plummer(3, 2048)
    pos = pm[:, :3].astype(np.float64)
    v = vel[:, :3].astype(np.float64)
    m = pm[:, 3].astype(np.float64)
    out = ref.app_steps(pos, v, m, np.zeros_like(pos), 1e-3, THETA, 1.0, 3)
    assert out["rc"] == 0
    np.savez_compressed(os.path.join(HERE, "literal_app_steps.npz"), pos_m=pm, vel=vel, dt=np.array([1e-3]),
                        theta=np.array([THETA]), steps=np.array([3]), out_pos=out["pos"], out_vel=out["vel"],
                        out_acc=out["acc"], out_perm=out["perm"])
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
