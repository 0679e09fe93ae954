"""The rule the all-depths tree build (k_nodes_count / k_nodes_write / k_nodes_link) rests on,
checked on the CPU against the oracle's top-down insertion build:

  * with the bodies in tree-key order, E(i) = max over j in [i - L, i] of the digits that keys
    j and j + L share is the deepest depth at which body i's cell holds more than L bodies;
  * a depth-d node starts at body i exactly for d from (digits shared with key i - 1) + 1 to
    min(E(i) + 1, 21), and it is internal exactly when d < min(E(i) + 1, 21);
  * its cell ends at the first later body whose key parts from its predecessor's within the
    first d digits (that body starts a node of depth d or less).
"""
import zlib

import numpy as np
import pytest

from oracle.oracle import Restatement

MAX_DEPTH = 21


def bit_length(x):
    x = x.astype(np.uint64).copy()
    n = np.zeros(x.shape, np.int64)
    for s in (32, 16, 8, 4, 2, 1):
        big = x >= (np.uint64(1) << np.uint64(s))
        n[big] += s
        x = np.where(big, x >> np.uint64(s), x)
    return n + (x > 0)


def common_digits(a, b):
    x = a ^ b
    return np.where(x == 0, MAX_DEPTH, (64 - bit_length(x) - 1) // 3)


def nodes_by_rule(keys, L):
    """(node keys, body counts, internal flags) of the tree over sorted tree keys, by the rule."""
    n = len(keys)
    lcp = np.full(n, -1, np.int64)
    lcp[1:] = common_digits(keys[:-1], keys[1:])
    w = np.full(n, -1, np.int64)
    if n > L:
        w[: n - L] = common_digits(keys[: n - L], keys[L:])
    e = np.full(n, -1, np.int64)
    for q in range(L + 1):  # E(i) = max of w(j) over j in [i - L, i]: shift s = L - q
        s = L - q
        if s < n:
            e[s:] = np.maximum(e[s:], w[: n - s])
    lo = np.maximum(lcp + 1, 1)
    hi = np.minimum(e + 1, MAX_DEPTH)
    out_keys, out_counts, out_internal = [1], [n], [n > L]
    idx = np.arange(n)
    for d in range(1, MAX_DEPTH + 1):
        starts = idx[(lo <= d) & (d <= hi)]
        bounds = idx[lo <= d]  # bodies whose key parts from the previous one within d digits
        nxt = np.searchsorted(bounds, starts, side="right")
        ends = np.where(nxt < len(bounds), bounds[np.minimum(nxt, len(bounds) - 1)], n)
        out_keys += list((keys[starts] >> np.uint64(3 * (MAX_DEPTH - d))).tolist())
        out_counts += list((ends - starts).tolist())
        out_internal += list((d < hi[starts]).tolist())
    order = np.argsort(np.array(out_keys, np.uint64), kind="stable")
    return (np.array(out_keys, np.uint64)[order], np.array(out_counts, np.int64)[order],
            np.array(out_internal)[order])


def sorted_scene(pos, edge_factor=2.0):
    orc = Restatement()
    c, size = orc.bounds(pos)
    edge = edge_factor * size
    keys = orc.tree_keys(pos, c, edge)
    order = np.argsort(keys, kind="stable")
    return orc, pos[order], np.asarray(keys)[order].astype(np.uint64), c, edge


TINY = {1: 2, 3: 5, 16: 4}  # fewer bodies than, or about, the leaf capacity


@pytest.mark.parametrize("case", ["gauss", "clustered", "coincident", "tiny"])
@pytest.mark.parametrize("leaf", [1, 3, 16])
def test_all_depths_rule_matches_insertion_build(case, leaf):
    rng = np.random.default_rng(zlib.crc32(f"{case}/{leaf}".encode()))
    if case == "gauss":
        pos = rng.normal(size=(6000, 3))
    elif case == "clustered":
        centres = rng.uniform(-50, 50, size=(12, 3))
        pos = centres[rng.integers(0, 12, 6000)] + rng.normal(scale=1e-3, size=(6000, 3))
    elif case == "coincident":
        pos = rng.uniform(-1, 1, size=(3000, 3))
        pos[1000:1030] = pos[7]  # a bucket at depth 21
    else:
        pos = rng.uniform(-1, 1, size=(TINY[leaf], 3))
    pos = pos.astype(np.float32).astype(np.float64)
    orc, spos, keys, c, edge = sorted_scene(pos)
    mass = np.full(len(spos), 1.0 / len(spos))
    want = orc.build(spos, mass, c, edge, leaf, 1)
    got_keys, got_counts, got_internal = nodes_by_rule(keys, leaf)
    assert np.array_equal(got_keys, want["keys"].astype(np.uint64))
    assert np.array_equal(got_counts, want["counts"])
    assert np.array_equal(got_internal, want["child_byte"] != 0)
