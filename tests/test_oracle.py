"""The oracle restatement, pinned against REF-LITERAL (the reference's own compiled code).

Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from REF-LITERAL) pin
it everywhere; where the reference checkout exists the tests also run REF-LITERAL live on
fresh seeds.
"""
import numpy as np
import pytest

from conftest import golden
from oracle.oracle import relerr

SMALL = None


def small_cases():
    global SMALL
    if SMALL is None:
        d = golden("literal_small.npz")
        names = sorted({k.split("/")[0] for k in d.files})
        SMALL = (d, names)
    return SMALL


def case_names():
    return small_cases()[1]


@pytest.mark.parametrize("name", case_names())
def test_restatement_matches_golden_small(orc, name):
    d, _ = small_cases()
    g = lambda k: d[f"{name}/{k}"]  # noqa: E731
    pm = g("pos_m")
    pos = pm[:, :3].astype(np.float64)
    mass = pm[:, 3].astype(np.float64)
    c, size = orc.bounds(pos)
    assert np.array_equal(c, g("center")) and size == g("size")[0]
    keys = orc.morton_keys(pos, size)
    assert np.array_equal(keys, g("keys"))
    perm = orc.sort_perm(keys)
    assert np.array_equal(perm, g("perm"))
    sp, sm = pos[perm], mass[perm]
    for tag, ef in (("e1", 1.0), ("e2", 2.0)):
        if f"{name}/{tag}_refused" in d.files:
            assert size <= 0 or orc.guard(sp, c, size * ef) > 0
            continue
        assert orc.guard(sp, c, size * ef) == 0
        t = orc.build(sp, sm, c, size * ef, 1, 0)
        assert np.array_equal(t["keys"], g(f"{tag}_node_keys"))
        assert np.array_equal(t["counts"], g(f"{tag}_node_counts"))
        assert np.array_equal(t["child_byte"], g(f"{tag}_node_child"))
        assert np.array_equal(t["com"], g(f"{tag}_node_com"))
        assert np.array_equal(t["mass"], g(f"{tag}_node_mass"))
        acc, nc, npp = orc.force(sp, sm, c, size * ef, 1, 0, 0.5, 0.025)
        assert np.array_equal(nc + npp, g(f"{tag}_list_len"))
        # same FP64 operations in the same order: bit-identical
        assert np.array_equal(acc, g(f"{tag}_acc"))


def test_restatement_matches_golden_config0(orc):
    d = golden("literal_config0.npz")
    pm = d["pos_m"]
    pos = pm[:, :3].astype(np.float64)
    mass = pm[:, 3].astype(np.float64)
    c, size = orc.bounds(pos)
    assert np.array_equal(c, d["center"]) and size == d["size"][0]
    keys = orc.morton_keys(pos, size)
    assert np.array_equal(keys, d["keys"])
    perm = orc.sort_perm(keys)
    assert np.array_equal(perm, d["perm"])
    sp, sm = pos[perm], mass[perm]
    assert orc.guard(sp, c, size) == 0
    t = orc.build(sp, sm, c, size, 1, 0)
    assert np.array_equal(t["keys"], d["e1_node_keys"])
    assert np.array_equal(t["counts"], d["e1_node_counts"])
    acc, nc, npp = orc.force(sp, sm, c, size, 1, 0, 0.5, 0.025, nthreads=4)
    assert np.array_equal(nc + npp, d["e1_list_len"])
    assert np.max(relerr(acc, d["e1_acc"])) < 1e-6  # fixture stored in FP32


def test_restatement_matches_golden_app_steps(orc):
    d = golden("literal_app_steps.npz")
    pm, vel = d["pos_m"], d["vel"]
    out = orc.steps(pm[:, :3], vel[:, :3], pm[:, 3], np.zeros((len(pm), 3)), float(d["dt"][0]),
                    float(d["theta"][0]), 0.025, 1.0, 1, 0, int(d["steps"][0]), acc_follows_body=0)
    assert np.array_equal(out["perm"], d["out_perm"])
    assert np.array_equal(out["pos"], d["out_pos"])
    assert np.array_equal(out["vel"], d["out_vel"])
    assert np.array_equal(out["acc"], d["out_acc"])


@pytest.mark.parametrize("seed,n,ef", [(11, 3000, 1.0), (12, 5000, 2.0)])
def test_restatement_matches_ref_live(bh, orc, ref, seed, n, ef):
    pm, _ = bh.plummer(seed, n)
    pos = pm[:, :3].astype(np.float64)
    mass = pm[:, 3].astype(np.float64)
    c, size = ref.bounds(pos)
    c2, size2 = orc.bounds(pos)
    assert np.array_equal(c, c2) and size == size2
    keys = ref.morton_keys(pos, size)
    assert np.array_equal(keys, orc.morton_keys(pos, size))
    perm = ref.sort_perm(keys)
    assert np.array_equal(perm, orc.sort_perm(keys))
    sp, sm = pos[perm], mass[perm]
    edge = size * ef
    assert ref.guard(sp, c, edge) == orc.guard(sp, c, edge) == 0
    t_ref = ref.build(sp, sm, c, edge)
    t = orc.build(sp, sm, c, edge, 1, 0)
    for k in ("keys", "counts", "child_byte", "com", "mass"):
        assert np.array_equal(t[k], t_ref[k]), k
    a_ref, ll = ref.force(sp, sm, c, edge, 0.5)
    a, nc, npp = orc.force(sp, sm, c, edge, 1, 0, 0.5, 0.025)
    assert np.array_equal(a, a_ref)
    assert np.array_equal(nc + npp, ll)


def test_guard_detects_shared_depth21_cell(orc, ref):
    pos = np.array([[0.1, 0.2, 0.3], [0.1, 0.2, 0.3], [-0.5, 0.5, 0.5]])
    assert orc.guard(pos, np.zeros(3), 2.0) == 1
    assert ref.guard(pos, np.zeros(3), 2.0) == 1


def test_intended_upsweep_matches_direct_moments(orc):
    """Intended mode: node mass / COM / quadrupole equal the direct sums over member bodies."""
    rng = np.random.default_rng(5)
    n = 300
    pos = rng.normal(size=(n, 3))
    mass = rng.uniform(0.5, 1.5, n) / n
    t = orc.build(pos, mass, np.zeros(3), 16.0, 4, 1)
    tk = orc.tree_keys(pos, np.zeros(3), 16.0)
    for j in range(0, len(t["keys"]), 7):
        key = int(t["keys"][j])
        depth = (key.bit_length() - 1) // 3
        members = (tk >> np.uint64(3 * (21 - depth))) == np.uint64(key)
        m = mass[members]
        x = pos[members]
        com = (m[:, None] * x).sum(0) / m.sum()
        assert t["counts"][j] == members.sum()
        assert np.isclose(t["mass"][j], m.sum(), rtol=1e-13)
        assert np.allclose(t["com"][j], com, rtol=1e-10, atol=1e-12)
        r = x - com
        r2 = (r * r).sum(1)
        q = np.array([(m * (3 * r[:, a] * r[:, b] - (a == b) * r2)).sum()
                      for a, b in ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))])
        assert np.allclose(t["quad"][j], q, rtol=1e-9, atol=1e-12)


def test_intended_force_close_to_direct_sum(orc):
    """REF-INTENDED's own accuracy at theta = 0.5 against the FP64 direct sum."""
    import __graft_entry__

    bh = __graft_entry__.package()
    pm, _ = bh.plummer(1, 8192)
    pos = pm[:, :3].astype(np.float64)
    mass = pm[:, 3].astype(np.float64)
    c, size = orc.bounds(pos)
    a, _, _ = orc.force(pos, mass, c, 2 * size, 1, 1, 0.5, 0.01, nthreads=4)
    d = orc.direct(pos, mass, 0.01, nthreads=4)
    err = relerr(a, d)
    assert np.median(err) < 1e-3
    lit, _, _ = orc.force(pos, mass, c, 2 * size, 1, 0, 0.5, 0.01, nthreads=4)
    assert np.median(relerr(lit, d)) > 1e-2  # the literal pseudo-barycentre walk is far less accurate


def test_decode_morton_matches_reference(orc, ref):
    """decodeMortonKey: the restatement equals the reference's own function bit for bit, on keys
    of real positions and on arbitrary 64-bit words (the decode ignores bit 63 and reads every
    axis bit)."""
    rng = np.random.default_rng(8)
    pos = rng.normal(0, 2, (5000, 3))
    c, size = orc.bounds(pos)
    keys = np.concatenate([orc.morton_keys(pos, size), rng.integers(0, 2**63, 3000, dtype=np.uint64) | (1 << 63)])
    for s in (size, 1.0, 3.75e11):
        assert np.array_equal(orc.decode_morton(keys, s), ref.decode_morton(keys, s))
    # a key decodes to its cell's low corner: within one cell of the encoded position
    dec = orc.decode_morton(keys[:5000], size)
    assert np.all(np.abs(dec - pos) <= 2 * size / 2**21 * (1 + 1e-12))


def boxes_from_keys(keys, center, edge):
    """Each node's cube from its key alone, by the child-bounds recurrence (FP64, one rounding
    per operation: size' = size * 0.5; c' = c + (+-0.5) * size'), vectorised over the nodes."""
    keys = np.asarray(keys, np.uint64)
    depth = np.array([(int(k).bit_length() - 1) // 3 for k in keys])
    c = np.tile(np.asarray(center, np.float64), (len(keys), 1))
    s = np.full(len(keys), float(edge))
    for lvl in range(int(depth.max(initial=0))):
        live = depth > lvl  # nodes below level lvl take the step to their level-(lvl + 1) ancestor
        shift = (3 * (depth - lvl - 1)).clip(min=0).astype(np.uint64)
        o = ((keys >> shift) & np.uint64(7)).astype(np.int64)
        s = np.where(live, s * 0.5, s)
        for a in range(3):
            half = np.where((o >> (2 - a)) & 1, 0.5, -0.5)
            c[:, a] = np.where(live, c[:, a] + half * s, c[:, a])
    return np.column_stack([c, s]), depth


@pytest.mark.parametrize("name", sorted({k.split("/")[0] for k in golden("literal_small.npz").files}))
def test_node_boxes_golden_follow_child_recurrence(name):
    """REF-LITERAL's nodeBounds (the cubes visualizeTree draws) are the child-bounds recurrence
    applied along each node key from the root cube, bit for bit: the rule bh_tree_boxes uses."""
    d = golden("literal_small.npz")
    for tag, ef in (("e1", 1.0), ("e2", 2.0)):
        if f"{name}/{tag}_refused" in d.files:
            continue
        box, _ = boxes_from_keys(d[f"{name}/{tag}_node_keys"], d[f"{name}/center"], d[f"{name}/size"][0] * ef)
        assert np.array_equal(box, d[f"{name}/{tag}_node_box"]), (name, tag)


def test_node_boxes_golden_config0_follow_child_recurrence():
    d = golden("literal_config0.npz")
    box, _ = boxes_from_keys(d["e1_node_keys"], d["center"], d["size"][0])
    assert np.array_equal(box.astype(np.float32), d["e1_node_box"])
