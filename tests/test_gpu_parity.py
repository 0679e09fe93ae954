"""GPU parity: libbhgpu (through its C ABI) against the oracle and the REF-LITERAL golden vectors.

Bars:
  * bounds size, Morton keys, sort permutation, node-key set, node body counts and child
    bytes, literal pseudo-barycentres, node cubes (FP64 nodeBounds rounded to FP32): bit-exact;
  * accelerations against the reference walk at the same theta, softening and leaf size:
    median relative error <= 1e-5 and 99th percentile <= 1e-4 (FP32 kernel vs FP64 oracle);
  * accelerations against the FP64 direct sum at theta = 0.5: median <= 1e-3.
"""
import numpy as np
import pytest

from conftest import golden
from oracle.oracle import relerr

pytestmark = pytest.mark.gpu

MED, P99 = 1e-5, 1e-4


def assert_acc_close(acc, ref, med=MED, p99=P99):
    err = relerr(acc, ref)
    m, p = float(np.median(err)), float(np.percentile(err, 99))
    assert m <= med and p <= p99, f"median {m:.3e} p99 {p:.3e}"
    return m, p


@pytest.fixture(scope="module")
def sim(bh):
    s = bh.Simulation(1 << 21)
    yield s
    s.close()


def small_cases():
    d = golden("literal_small.npz")
    return d, sorted({k.split("/")[0] for k in d.files})


@pytest.mark.parametrize("name", small_cases()[1])
def test_literal_small_cases_vs_golden(bh, sim, name):
    d, _ = small_cases()
    g = lambda k: d[f"{name}/{k}"]  # noqa: E731
    pm = g("pos_m")
    sim.set_bodies(pm, np.zeros_like(pm))
    c, size = sim.bounds()
    assert size == g("size")[0]
    assert np.allclose(c, g("center"), rtol=1e-14, atol=1e-300)
    keys = sim.morton_keys(size)
    assert np.array_equal(keys, g("keys"))
    perm = sim.sort_bodies()
    assert np.array_equal(perm, g("perm"))
    for tag, ef in (("e1", 1.0), ("e2", 2.0)):
        if f"{name}/{tag}_refused" in d.files:
            continue
        sim.build(g("center"), size * ef, 1, bh.BH_MULTIPOLE_LITERAL)
        t = sim.tree_nodes()
        assert np.array_equal(t["keys"], g(f"{tag}_node_keys"))
        assert np.array_equal(t["counts"], g(f"{tag}_node_counts"))
        assert np.array_equal(t["child_byte"], g(f"{tag}_node_child"))
        assert np.array_equal(t["com"], g(f"{tag}_node_com"))
        assert np.allclose(t["mass"], g(f"{tag}_node_mass"), rtol=1e-12)
        # node cubes (visualizeTree's boxes): the reference's FP64 nodeBounds rounded to FP32
        box, _, count = sim.tree_boxes()
        assert np.array_equal(box, g(f"{tag}_node_box").astype(np.float32))
        assert np.array_equal(count, g(f"{tag}_node_counts"))
        acc, st = sim.force(0.5, 0.025, stats=True)
        if len(pm) > 1:
            assert_acc_close(acc, g(f"{tag}_acc"))
        else:
            assert np.all(acc == 0)
        assert st.interactions_p2p + st.interactions_cell == g(f"{tag}_list_len").sum()


def test_literal_config0_vs_golden(bh, sim):
    d = golden("literal_config0.npz")
    pm = d["pos_m"]
    sim.set_bodies(pm, np.zeros_like(pm))
    c, size = sim.bounds()
    assert size == d["size"][0]
    keys = sim.morton_keys(size)
    assert np.array_equal(keys, d["keys"])
    perm = sim.sort_bodies()
    assert np.array_equal(perm, d["perm"])
    sim.build(d["center"], size, 1, bh.BH_MULTIPOLE_LITERAL)
    t = sim.tree_nodes()
    assert np.array_equal(t["keys"], d["e1_node_keys"])
    assert np.array_equal(t["counts"], d["e1_node_counts"])
    assert np.array_equal(sim.tree_boxes()[0], d["e1_node_box"])
    acc, st = sim.force(0.5, 0.025, stats=True)
    assert_acc_close(acc, d["e1_acc"])
    assert abs(int(st.interactions_p2p) - int(d["e1_list_len"].sum())) <= 1e-4 * d["e1_list_len"].sum()


@pytest.mark.parametrize("leaf,theta", [(1, 0.5), (8, 0.5), (16, 0.3), (16, 0.5), (16, 0.7)])
def test_intended_force_vs_oracle(bh, orc, sim, leaf, theta):
    n = 20000
    pm, v = bh.plummer(21 + leaf, n)
    sim.set_bodies(pm, v)
    c, size = sim.bounds()
    sim.morton_keys(size)
    perm = sim.sort_bodies()
    sp = pm[perm]
    edge = 2 * size
    sim.build(c, edge, leaf, bh.BH_MULTIPOLE_QUADRUPOLE)
    t = sim.tree_nodes()
    pos = sp[:, :3].astype(np.float64)
    mass = sp[:, 3].astype(np.float64)
    ref_t = orc.build(pos, mass, c, edge, leaf, 1)
    assert np.array_equal(t["keys"], ref_t["keys"])
    assert np.array_equal(t["counts"], ref_t["counts"])
    assert np.array_equal(t["child_byte"], ref_t["child_byte"])
    # mass and centre of mass: float-float (~44 bits) against FP64
    assert np.allclose(t["mass"], ref_t["mass"], rtol=1e-11)
    assert np.allclose(t["com"], ref_t["com"], rtol=1e-9, atol=1e-12)
    # quadrupole: FP32, against its natural scale mass * edge^2 of the node
    depth = np.array([(int(k).bit_length() - 1) // 3 for k in t["keys"]])
    scale = ref_t["mass"] * (edge / 2.0 ** depth) ** 2
    assert np.all(np.abs(t["quad"] - ref_t["quad"]) <= 1e-5 * scale[:, None])
    acc, st = sim.force(theta, 0.005, stats=True)
    ref_acc, nc, npp = orc.force(pos, mass, c, edge, leaf, 1, theta, 0.005, nthreads=8)
    assert_acc_close(acc, ref_acc)
    assert abs(int(st.interactions_cell) - int(nc.sum())) <= 1e-4 * nc.sum() + 2
    assert abs(int(st.interactions_p2p) - int(npp.sum())) <= 1e-4 * npp.sum() + 2
    if theta == 0.5:
        tgt = np.arange(0, n, 7, dtype=np.uint32)
        direct = orc.direct(pos, mass, 0.005, targets=tgt, nthreads=8)
        assert np.median(relerr(acc[tgt], direct)) <= 1e-3


def test_literal_two_spheres_deep_tree(bh, orc, sim):
    """Clustered input: depths up to 21, uneven groups, bucket leaves allowed (L = 8)."""
    pm, v = bh.two_spheres(5, 40000)
    sim.set_bodies(pm, v)
    c, size = sim.bounds()
    sim.morton_keys(size)
    perm = sim.sort_bodies()
    sp = pm[perm]
    pos, mass = sp[:, :3].astype(np.float64), sp[:, 3].astype(np.float64)
    for mode in (bh.BH_MULTIPOLE_LITERAL, bh.BH_MULTIPOLE_QUADRUPOLE):
        sim.build(c, 2 * size, 8, mode)
        t = sim.tree_nodes()
        ref_t = orc.build(pos, mass, c, 2 * size, 8, mode)
        assert np.array_equal(t["keys"], ref_t["keys"])
        assert np.array_equal(t["counts"], ref_t["counts"])
        acc = sim.force(0.5, 0.001)
        ref_acc, _, _ = orc.force(pos, mass, c, 2 * size, 8, mode, 0.5, 0.001, nthreads=8)
        assert_acc_close(acc, ref_acc)


def test_coincident_bodies_bucket_at_depth21(bh, orc, sim):
    """Bodies sharing a depth-21 cell: the reference cannot build this (its key overflows);
    libbhgpu keeps them in one depth-21 leaf and sums them pairwise."""
    pm, v = bh.plummer(8, 3000)
    pm[1000:1010, :3] = pm[5, :3]
    pm[2000:2003, :3] = pm[7, :3] + np.float32(1e-7)
    sim.set_bodies(pm, v)
    c, size = sim.bounds()
    sim.morton_keys(size)
    perm = sim.sort_bodies()
    sp = pm[perm]
    pos, mass = sp[:, :3].astype(np.float64), sp[:, 3].astype(np.float64)
    assert orc.guard(pos, c, 2 * size) > 0
    sim.build(c, 2 * size, 1, bh.BH_MULTIPOLE_QUADRUPOLE)
    t = sim.tree_nodes()
    ref_t = orc.build(pos, mass, c, 2 * size, 1, 1)
    assert np.array_equal(t["keys"], ref_t["keys"])
    assert np.array_equal(t["counts"], ref_t["counts"])
    acc = sim.force(0.5, 0.01)
    ref_acc, _, _ = orc.force(pos, mass, c, 2 * size, 1, 1, 0.5, 0.01)
    assert_acc_close(acc, ref_acc)
    assert np.all(np.isfinite(acc))


# the sorts go by rank up to 16 384 keys (the radix sort beyond): the sizes either side of the
# limit take both paths
@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 1000, 1025, 4097, 8192, 8193, 16384, 16385])
def test_small_and_ragged_n(bh, orc, sim, n):
    pm, v = bh.plummer(300 + n, n)
    sim.set_bodies(pm, v)
    c, size = sim.bounds()
    pos = pm[:, :3].astype(np.float64)
    c2, size2 = orc.bounds(pos)
    assert size == size2
    if size <= 0:
        return
    keys = sim.morton_keys(size)
    assert np.array_equal(keys, orc.morton_keys(pos, size))
    perm = sim.sort_bodies()
    assert np.array_equal(perm, orc.sort_perm(keys))
    sp = pm[perm]
    p2, m2 = sp[:, :3].astype(np.float64), sp[:, 3].astype(np.float64)
    for leaf in (1, 16):
        sim.build(c, 2 * size, leaf, bh.BH_MULTIPOLE_QUADRUPOLE)
        assert np.array_equal(sim.tree_nodes()["keys"], orc.build(p2, m2, c, 2 * size, leaf, 1)["keys"])
        acc = sim.force(0.5, 0.01)
        ref_acc, _, _ = orc.force(p2, m2, c, 2 * size, leaf, 1, 0.5, 0.01)
        assert_acc_close(acc, ref_acc)


def test_node_lookup(bh, sim):
    pm, v = bh.plummer(17, 5000)
    sim.set_bodies(pm, v)
    c, size = sim.bounds()
    sim.build(c, 2 * size, 4, bh.BH_MULTIPOLE_QUADRUPOLE)
    t = sim.tree_nodes()
    rng = np.random.default_rng(0)
    for j in rng.choice(len(t["keys"]), 50, replace=False):
        nd = sim.lookup(t["keys"][j])
        assert nd.key == t["keys"][j] and nd.count == t["counts"][j] and nd.child_byte == t["child_byte"][j]
        assert np.allclose(nd.com[:], t["com"][j])
        assert nd.depth == (int(t["keys"][j]).bit_length() - 1) // 3
        assert np.isclose(nd.size, 2 * size / 2 ** nd.depth)
    root = sim.lookup(1)
    assert root.count == 5000 and root.depth == 0
    with pytest.raises(bh.BHError) as e:
        sim.lookup((1 << 60) | 12345)
    assert e.value.code == 9


@pytest.mark.parametrize("leaf", [1, 8, 64, 65, 200])
def test_build_paths_by_leaf_capacity(bh, orc, sim, leaf):
    """Leaf capacities up to 64 build every depth at once, larger ones level by level; both give
    the reference's node set, counts and child bytes."""
    n = 20000
    pm, v = bh.plummer(77, n)
    pm[5000:5040, :3] = pm[11, :3]  # a run of coincident bodies: a bucket at depth 21
    sim.set_bodies(pm, v)
    c, size = sim.bounds()
    sim.morton_keys(size)
    perm = sim.sort_bodies()
    sp = pm[perm]
    pos, mass = sp[:, :3].astype(np.float64), sp[:, 3].astype(np.float64)
    sim.build(c, 2 * size, leaf, bh.BH_MULTIPOLE_QUADRUPOLE)
    t = sim.tree_nodes()
    ref_t = orc.build(pos, mass, c, 2 * size, leaf, 1)
    assert np.array_equal(t["keys"], ref_t["keys"])
    assert np.array_equal(t["counts"], ref_t["counts"])
    assert np.array_equal(t["child_byte"], ref_t["child_byte"])
    acc = sim.force(0.5, 0.01)
    ref_acc, _, _ = orc.force(pos, mass, c, 2 * size, leaf, 1, 0.5, 0.01, nthreads=8)
    assert_acc_close(acc, ref_acc)


def test_node_arena_growth(bh, orc, sim):
    """Tight pairs make long single-child chains: more nodes than the initial arena holds."""
    rng = np.random.default_rng(3)
    base = rng.uniform(-1, 1, (600, 3))
    pos = np.concatenate([base, base + 1e-6 * rng.uniform(-1, 1, (600, 3))]).astype(np.float32)
    pm = np.zeros((1200, 4), np.float32)
    pm[:, :3] = pos
    pm[:, 3] = 1.0 / 1200
    sim.set_bodies(pm, np.zeros_like(pm))
    c, size = sim.bounds()
    sim.build(c, 2 * size, 1, bh.BH_MULTIPOLE_QUADRUPOLE)
    t = sim.tree_nodes()
    ref_t = orc.build(pos.astype(np.float64), pm[:, 3].astype(np.float64), c, 2 * size, 1, 1)
    assert len(t["keys"]) > 2 * 1200 + 64
    assert np.array_equal(t["keys"], ref_t["keys"])


def test_step_matches_oracle_step(bh, orc, sim):
    """One fused bh_step against the oracle's step (same inputs, same order of stages)."""
    n = 30000
    pm, v = bh.plummer(2, n)
    v[:, 3] = np.arange(n, dtype=np.float32)  # body id rides in the unused velocity lane
    acc0 = np.zeros((n, 4), np.float32)
    acc0[:, :3] = np.random.default_rng(1).normal(scale=0.1, size=(n, 3)).astype(np.float32)
    sim.set_bodies(pm, v, acc0)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=8, edge_factor=2.0)
    st = sim.step(prm, 1)
    assert st.steps == 1 and st.error_flags == 0
    p1, v1, a1 = sim.get_bodies()
    out = orc.steps(pm[:, :3], v[:, :3], pm[:, 3], acc0[:, :3], 1e-3, 0.5, 0.01, 2.0, 8, 1, 1,
                    acc_follows_body=1, nthreads=8)
    # the Morton sort ran on identical inputs: same permutation
    assert np.array_equal(v1[:, 3].astype(np.int64), out["perm"].astype(np.int64))
    assert np.allclose(p1[:, :3], out["pos"], rtol=0, atol=1e-6)
    assert np.allclose(v1[:, :3], out["vel"], rtol=0, atol=1e-6)
    assert_acc_close(a1, out["acc"])


def test_step_reference_app_order_vs_golden(bh, sim):
    """Three frames in the app's order (literal multipoles, edge S, acceleration array not
    reordered by the sort) against REF-LITERAL's own frames."""
    d = golden("literal_app_steps.npz")
    pm, vel = d["pos_m"].copy(), d["vel"].copy()
    n = len(pm)
    vel[:, 3] = np.arange(n, dtype=np.float32)
    sim.set_bodies(pm, vel)
    prm = bh.default_params(theta=float(d["theta"][0]), eps=0.025, dt=float(d["dt"][0]), leaf_capacity=1,
                            multipole=bh.BH_MULTIPOLE_LITERAL, edge_factor=1.0, acc_follows_body=0)
    sim.step(prm, int(d["steps"][0]))
    p, v, a = sim.get_bodies()
    ids = v[:, 3].astype(np.int64)
    ref_ids = d["out_perm"].astype(np.int64)
    same = ids == ref_ids
    assert same.mean() > 0.999  # a body near a key boundary may sort differently after FP32 steps
    assert np.allclose(p[same, :3], d["out_pos"][same], rtol=0, atol=1e-5)
    assert np.allclose(v[same, :3], d["out_vel"][same], rtol=0, atol=1e-4)


def test_piecewise_leapfrog_halves(bh, sim):
    n = 1000
    pm, v = bh.plummer(4, n)
    acc = np.zeros((n, 4), np.float32)
    acc[:, :3] = np.random.default_rng(2).normal(size=(n, 3)).astype(np.float32)
    sim.set_bodies(pm, v, acc)
    sim.kick_drift(0.01)
    p, vv, _ = sim.get_bodies()
    v_half = v[:, :3] + acc[:, :3] * np.float32(0.005)
    assert np.allclose(vv[:, :3], v_half, atol=1e-6)
    assert np.allclose(p[:, :3], pm[:, :3] + v_half * np.float32(0.01), atol=1e-6)
    sim.kick(0.01)
    _, v2, _ = sim.get_bodies()
    assert np.allclose(v2[:, :3], v_half + acc[:, :3] * np.float32(0.005), atol=1e-6)


def test_reference_body_layout_roundtrip(bh, sim):
    n = 257
    pm, v = bh.plummer(6, n)
    rec = np.zeros(n, dtype=[("color", "u1", 8), ("radius", "f8"), ("pos", "f8", 3), ("vel", "f8", 3),
                             ("mass", "f8"), ("key", "u8")])
    assert rec.dtype.itemsize == 80
    rec["pos"] = pm[:, :3]
    rec["vel"] = v[:, :3]
    rec["mass"] = pm[:, 3]
    rec["radius"] = 7.0
    lib = bh.load()
    bh.check(lib.bh_set_bodies_ref(sim.h, rec.ctypes.data, n), "set_ref")
    c, size = sim.bounds()
    keys = sim.morton_keys(size)
    sim.sort_bodies()
    out = rec.copy()
    bh.check(lib.bh_get_bodies_ref(sim.h, out.ctypes.data, n), "get_ref")
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(out["key"], keys[order])
    assert np.array_equal(out["pos"], rec["pos"][order].astype(np.float32).astype(np.float64))
    assert np.all(out["radius"] == 7.0)


def test_full_size_keys_perm_nodes(bh, orc):
    """N = 2^22 (the at-scale Plummer size): keys, permutation and node set bit-exact; step-0
    forces against the reference's tree walk (the oracle, same theta, softening and leaf size) on
    a seeded 65 536-body subsample at theta 0.5 and 8192 bodies at theta 0.3 and 0.7, and against
    the FP64 direct sum."""
    n = 1 << 22
    pm, v = bh.plummer(0, n)
    pos = pm[:, :3].astype(np.float64)
    with bh.Simulation(n) as s:
        s.set_bodies(pm, v)
        c, size = s.bounds()
        c2, size2 = orc.bounds(pos)
        assert size == size2 and np.allclose(c, c2, rtol=1e-12, atol=1e-18)
        keys = s.morton_keys(size)
        assert np.array_equal(keys, orc.morton_keys(pos, size))
        perm = s.sort_bodies()
        assert np.array_equal(perm, orc.sort_perm(keys))
        sp = pm[perm]
        p2, m2 = sp[:, :3].astype(np.float64), sp[:, 3].astype(np.float64)
        s.build(c, 2 * size, 16, bh.BH_MULTIPOLE_QUADRUPOLE)
        t = s.tree_nodes()
        assert np.array_equal(t["keys"], orc.build(p2, m2, c, 2 * size, 16, 1)["keys"])
        for theta, ntgt in ((0.5, 65536), (0.3, 8192), (0.7, 8192)):
            acc = s.force(theta, 0.005)
            tgt = np.sort(np.random.default_rng(0).choice(n, ntgt, replace=False)).astype(np.uint32)
            ref_acc, _, _ = orc.force(p2, m2, c, 2 * size, 16, 1, theta, 0.005, targets=tgt, nthreads=16)
            assert_acc_close(acc[tgt], ref_acc)
            if theta == 0.5:
                direct = orc.direct(p2, m2, 0.005, targets=tgt[:512], nthreads=16)
                assert np.median(relerr(acc[tgt[:512]], direct)) <= 1e-3


def _near_boundaries(rng, n, points):
    """Float32 coordinates on, and 1 ulp either side of, the given FP64 boundary points."""
    x = rng.choice(points, n).astype(np.float32)
    side = rng.integers(-1, 2, n)
    x = np.where(side > 0, np.nextafter(x, np.float32(np.inf)), x)
    x = np.where(side < 0, np.nextafter(x, np.float32(-np.inf)), x)
    return x


@pytest.mark.parametrize("S,center,edge", [(1.0, (0.0, 0.0, 0.0), 2.0),
                                           (0.7734375, (0.1, -0.3, 0.05), 2.6),
                                           (3.3, (-1.25, 0.5, 2.0), 7.0)])
def test_key_fast_paths_at_cell_boundaries(bh, orc, sim, S, center, edge):
    """Morton and tree keys of coordinates sitting exactly on, or one float32 ulp beside, the
    cell boundaries of the key grids (and some outside the cube): the FP32 fast paths must hand
    every such coordinate to the exact FP64 path, so keys and the node set stay bit-exact."""
    rng = np.random.default_rng(11)
    n = 30000
    frac = 2.0 ** 21 / (2.0 * S)
    k = np.arange(-(1 << 21), (1 << 22) + 1, 97, dtype=np.float64)
    morton_pts = k / frac - S  # (p + S) * frac = k
    pm = np.zeros((n, 4), np.float32)
    for a in range(3):
        pm[:, a] = _near_boundaries(rng, n, morton_pts)
    pm[:, 3] = rng.uniform(0.5, 1.5, n) / n
    v = np.zeros_like(pm)
    sim.set_bodies(pm, v)
    keys = sim.morton_keys(S)
    assert np.array_equal(keys, orc.morton_keys(pm[:, :3].astype(np.float64), S))
    # tree-key comparison points: c0 + (k - 2^20) * edge / 2^21, k in [1, 2^21 - 1]
    kt = np.arange(-64, (1 << 21) + 64, 61, dtype=np.float64)
    for a in range(3):
        pm[:, a] = _near_boundaries(rng, n, center[a] + (kt - 2.0 ** 20) * edge / 2.0 ** 21)
    sim.set_bodies(pm, v)
    pos, mass = pm[:, :3].astype(np.float64), pm[:, 3].astype(np.float64)
    sim.build(np.array(center), edge, 4, bh.BH_MULTIPOLE_QUADRUPOLE)
    t = sim.tree_nodes()
    ref = orc.build(pos, mass, np.array(center), edge, 4, 1)
    assert np.array_equal(t["keys"], ref["keys"])
    assert np.array_equal(t["counts"], ref["counts"])


def test_decode_morton_keys_bit_exact(bh, orc, sim):
    """bh_decode_morton_keys against the oracle's decodeMortonKey restatement, bit for bit."""
    rng = np.random.default_rng(9)
    keys = np.concatenate([rng.integers(0, 2**63, 100000, dtype=np.uint64) | np.uint64(1 << 63),
                           np.array([1 << 63, (1 << 64) - 1, 0], np.uint64)])
    for size in (9.97, 1.0, 3.75e11):
        assert np.array_equal(sim.decode_morton_keys(keys, size), orc.decode_morton(keys, size))


def test_full_size_two_spheres(bh, orc):
    """Config 2 at full size (two Plummer spheres of 2^21, the deep-tree stress case): keys,
    permutation, node-key set and node counts bit-exact at leaf 8, and forces on a seeded
    subsample within the parity bars (theta 0.5, softening 0.001)."""
    n = 1 << 22
    pm, v = bh.two_spheres(0, n)
    pos = pm[:, :3].astype(np.float64)
    with bh.Simulation(n) as s:
        s.set_bodies(pm, v)
        c, size = s.bounds()
        keys = s.morton_keys(size)
        assert np.array_equal(keys, orc.morton_keys(pos, size))
        perm = s.sort_bodies()
        assert np.array_equal(perm, orc.sort_perm(keys))
        sp = pm[perm]
        p2, m2 = sp[:, :3].astype(np.float64), sp[:, 3].astype(np.float64)
        s.build(c, 2 * size, 8, bh.BH_MULTIPOLE_QUADRUPOLE)
        t = s.tree_nodes()
        ref_t = orc.build(p2, m2, c, 2 * size, 8, 1)
        assert np.array_equal(t["keys"], ref_t["keys"])
        assert np.array_equal(t["counts"], ref_t["counts"])
        assert (int(t["keys"][-1]).bit_length() - 1) // 3 >= 12  # the deepest level (14 here)
        acc = s.force(0.5, 0.001)
        tgt = np.random.default_rng(2).choice(n, 4096, replace=False).astype(np.uint32)
        ref_acc, _, _ = orc.force(p2, m2, c, 2 * size, 8, 1, 0.5, 0.001, targets=tgt, nthreads=16)
        assert_acc_close(acc[tgt], ref_acc)


def test_full_size_step_properties(bh):
    """Size-independent properties at N = 2^22: through fused steps the body ids riding in the
    velocity lane stay a permutation of 0..N-1 and the total mass is kept; a sort orders the
    keys and a second sort of the same keys is the identity."""
    n = 1 << 22
    pm, v = bh.plummer(3, n)
    v[:, 3] = np.arange(n, dtype=np.float32)
    prm = bh.default_params(theta=0.5, eps=0.005, dt=5e-4, leaf_capacity=16, multipole=1, edge_factor=2.0)
    with bh.Simulation(n) as s:
        s.set_bodies(pm, v)
        for _ in range(2):
            s.step(prm, 1)
            p, vv, _ = s.get_bodies()
            assert np.array_equal(np.sort(vv[:, 3].astype(np.int64)), np.arange(n))
            assert abs(float(p[:, 3].astype(np.float64).sum()) - float(pm[:, 3].astype(np.float64).sum())) < 1e-6
        # the drifted positions' keys: sorting orders them, and sorting again is the identity
        c, size = s.bounds()
        s.morton_keys(size)
        s.sort_bodies()
        again = s.sort_bodies()
        assert np.array_equal(again, np.arange(n, dtype=again.dtype))
        keys = s.morton_keys(size)
        assert np.all(keys[1:] >= keys[:-1])


def test_config0_trajectory_100_steps(bh, orc):
    """The small configuration run to its full length: N = 16 384 Plummer (seed 0), theta 0.5,
    eps 0.01, leaf 1, dt 1e-3, 100 KDK steps through bh_step (FP32) against the oracle's 100 steps
    (FP64, the reference's step order with intended multipoles), body by body (ids ride in the
    velocity lane): positions and velocities stay within FP32 drift of the FP64 trajectory."""
    n, nsteps = 16384, 100
    pm, v = bh.plummer(0, n)
    v[:, 3] = np.arange(n, dtype=np.float32)
    prm = bh.default_params(theta=0.5, eps=0.01, dt=1e-3, leaf_capacity=1, multipole=1, edge_factor=2.0)
    with bh.Simulation(n) as s:
        s.set_bodies(pm, v)
        st = s.step(prm, nsteps)
        assert st.steps == nsteps and st.error_flags == 0
        p, vv, _ = s.get_bodies()
    ids = vv[:, 3].astype(np.int64)
    assert np.array_equal(np.sort(ids), np.arange(n))
    out = orc.steps(pm[:, :3], v[:, :3], pm[:, 3], np.zeros((n, 3)), 1e-3, 0.5, 0.01, 2.0, 1, 1, nsteps,
                    acc_follows_body=1, nthreads=16)
    xo = np.empty((n, 3))
    vo = np.empty((n, 3))
    xo[out["perm"].astype(np.int64)] = out["pos"]
    vo[out["perm"].astype(np.int64)] = out["vel"]
    xg = np.empty((n, 3))
    vg = np.empty((n, 3))
    xg[ids] = p[:, :3]
    vg[ids] = vv[:, :3]
    dx = np.linalg.norm(xg - xo, axis=1)
    dv = np.linalg.norm(vg - vo, axis=1)
    print(f"config 0, 100 steps: |dx| median {np.median(dx):.2e} max {dx.max():.2e}; "
          f"|dv| median {np.median(dv):.2e} max {dv.max():.2e}")
    # measured: |dx| median 1.6e-7, max 8.9e-6; |dv| median 1.7e-7, max 3.9e-6
    assert np.median(dx) <= 1e-6 and dx.max() <= 1e-4
    assert np.median(dv) <= 1e-6 and dv.max() <= 1e-4
