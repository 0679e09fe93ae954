// CPU restatement of the reference's per-step Barnes-Hut path (the oracle).
//
// TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg load this library, as the checker or as the timed CPU baseline; the product
// (libbhgpu) never links or calls it.
//
// Written for this project from the reference's behaviour (no reference code is copied).
// Every function cites the reference lines it restates; file:line paths are relative to the
// reference project root. Two multipole semantics are provided:
//   mode 0 (literal)  : what the reference actually computes. Its upsweep never runs
//                       (insertBody nulls the caller's root pointer, src/HashedOctree.cpp:487,597,
//                       so ComputeHOTOctreeBaryCenters gets nullptr, src/HashedOctree.hpp:233 and
//                       returns at src/HashedOctree.cpp:831). Each node keeps the position of the
//                       first body inserted into it as its "barycentre", its mass is the running
//                       sum of inserted masses, and every quadrupole stays 0.
//   mode 1 (intended) : the reference's upsweep formulas (src/HashedOctree.cpp:721-855) run from
//                       the real root, without the nested leaf-zeroing recursion (:739), dividing
//                       by the mass once after the loop instead of inside it (:755). Bucket leaves
//                       (leaf capacity L > 1) treat their member bodies as single-body children.
// Arithmetic is FP64 throughout, like the reference's Vec3D (src/MathUtils.hpp:23-73).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <functional>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

constexpr int kMaxDepth = 21;  // 21 bits per axis: src/MortonKeys.hpp:42

// Vec3D::operator/= multiplies by the reciprocal and skips a zero divisor (src/MathUtils.cpp:81-90).
inline void div_by(double v[3], double s) {
  if (s != 0) {
    double inv = 1 / s;
    v[0] = v[0] * inv;
    v[1] = v[1] * inv;
    v[2] = v[2] * inv;
  }
}

// DetermineOctant: strict '>' per axis, x in bit 2 (src/OctantUtils.hpp:64-70).
inline int octant_of(const double c[3], const double p[3]) {
  return ((p[0] > c[0]) << 2) | ((p[1] > c[1]) << 1) | (int)(p[2] > c[2]);
}

// Child bounds of the HOTNode child constructor (src/HashedNode.cpp:48-70):
// size' = size * 0.5, centre' = centre + (dir * 0.5) * size'.
inline void child_bounds(const double c[3], double s, int oct, double cc[3], double* cs) {
  double half = s * 0.5;
  for (int a = 0; a < 3; ++a) {
    double dir = ((oct >> (2 - a)) & 1) ? 1.0 : -1.0;
    cc[a] = c[a] + (dir * 0.5) * half;
  }
  *cs = half;
}

// Magic-bit interleave of src/MortonKeys.hpp:95-124 (masks :51-58), applied to the full
// 64-bit coordinate words so out-of-range coordinates wrap exactly as in the reference.
inline uint64_t spread_bits(uint64_t v) {
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

// The reference converts the scaled coordinate with a plain (uint64_t) cast
// (src/MortonKeys.hpp:162-164), which C++ leaves undefined for negative or out-of-range values.
// The oracle pins what x86-64 gcc emits for it: below 2^63 (or NaN) a signed truncation with
// 0x8000000000000000 for NaN or values below -2^63; at or above 2^63 a truncation of x - 2^63
// with the top bit flipped, which is 0 for +inf and values of 2^64 or more.
inline uint64_t x86_trunc_u64(double x) {
  if (!(x >= 0x1p63)) {
    if (x >= -0x1p63) return (uint64_t)(int64_t)x;
    return 0x8000000000000000ull;
  }
  double y = x - 0x1p63;
  if (y < 0x1p63) return (uint64_t)(int64_t)y ^ 0x8000000000000000ull;
  return 0;
}

struct Node {
  double c[3];
  double size;
  double mass = 0;
  long n = 0;
  uint8_t child = 0;
  int depth = 0;
  double com[3] = {0, 0, 0};
  double q[6] = {0, 0, 0, 0, 0, 0};
  std::vector<uint32_t> members;  // leaf members in insertion order
};

using NodeMap = std::unordered_map<uint64_t, Node>;

// Top-down insertion with leaf capacity L, restating insertBody / pushHOTNodeBodyToChild /
// processNodeInsertion / createChildNode (src/HashedOctree.cpp:450-711). For L = 1 this is the
// reference's own rule: a leaf holding one body pushes it to a child when a second arrives.
// A leaf at depth 21 keeps any number of bodies (the reference has no such case: its key
// would overflow, which the guard rules out).
void insert_all(NodeMap& nodes, const double* pos3, const double* mass, size_t n, const double c0[3], double edge,
                int L) {
  nodes.clear();
  nodes.reserve(n * 2 + 16);
  Node& root = nodes[1];
  std::memcpy(root.c, c0, sizeof(root.c));
  root.size = edge;
  auto add_to_leaf = [&](Node& nd, uint32_t b) {
    if (nd.n == 0) std::memcpy(nd.com, pos3 + 3 * b, sizeof(nd.com));
    nd.n += 1;
    nd.mass = nd.mass + mass[b];
    nd.members.push_back(b);
  };
  for (size_t i = 0; i < n; ++i) {
    uint64_t key = 1;
    const double* p = pos3 + 3 * i;
    for (;;) {
      Node& nd = nodes[key];
      bool leaf = nd.child == 0;
      if (leaf && (nd.n < L || nd.depth == kMaxDepth)) {
        add_to_leaf(nd, (uint32_t)i);
        break;
      }
      if (leaf) {  // full leaf: push its members down before descending
        std::vector<uint32_t> mem;
        mem.swap(nd.members);
        double pc[3];
        std::memcpy(pc, nd.c, sizeof(pc));
        double ps = nd.size;
        int pd = nd.depth;
        for (uint32_t b : mem) {
          int o = octant_of(pc, pos3 + 3 * b);
          uint64_t ck = (key << 3) | (uint64_t)o;
          nodes[key].child |= (uint8_t)(1u << o);
          auto it = nodes.find(ck);
          if (it == nodes.end()) {
            Node ch;
            child_bounds(pc, ps, o, ch.c, &ch.size);
            ch.depth = pd + 1;
            it = nodes.emplace(ck, std::move(ch)).first;
          }
          add_to_leaf(it->second, b);
        }
      }
      Node& cur = nodes[key];
      cur.n += 1;
      cur.mass = cur.mass + mass[i];
      int o = octant_of(cur.c, p);
      uint64_t ck = (key << 3) | (uint64_t)o;
      if (cur.child & (1u << o)) {
        key = ck;
        continue;
      }
      cur.child |= (uint8_t)(1u << o);
      Node ch;
      child_bounds(cur.c, cur.size, o, ch.c, &ch.size);
      ch.depth = cur.depth + 1;
      auto it = nodes.emplace(ck, std::move(ch)).first;
      add_to_leaf(it->second, (uint32_t)i);
      break;
    }
  }
}

// Intended upsweep (see the file header). Post-order over children in octant order.
void upsweep(NodeMap& nodes, uint64_t key, const double* pos3, const double* mass) {
  Node& nd = nodes[key];
  if (nd.child == 0) {
    if (nd.n <= 1) return;  // single-body leaf keeps its body (src/HashedOctree.cpp:831)
    double m = 0, cm[3] = {0, 0, 0};
    for (uint32_t b : nd.members) {
      m += mass[b];
      for (int a = 0; a < 3; ++a) cm[a] += pos3[3 * b + a] * mass[b];
    }
    div_by(cm, m);
    nd.mass = m;
    std::memcpy(nd.com, cm, sizeof(cm));
    std::fill(nd.q, nd.q + 6, 0.0);
    for (uint32_t b : nd.members) {
      double x = pos3[3 * b] - cm[0], y = pos3[3 * b + 1] - cm[1], z = pos3[3 * b + 2] - cm[2];
      double mm = mass[b];
      nd.q[1] += 3.0 * mm * (x * y);
      nd.q[2] += 3.0 * mm * (x * z);
      nd.q[4] += 3.0 * mm * (y * z);
      double xx = x * x, yy = y * y, zz = z * z;
      double d2 = (xx + yy + zz) * mm;
      double m3 = mm * 3.0;
      nd.q[0] += m3 * xx - d2;
      nd.q[3] += m3 * yy - d2;
      nd.q[5] += m3 * zz - d2;
    }
    return;
  }
  for (int o = 0; o < 8; ++o)
    if (nd.child & (1u << o)) upsweep(nodes, (key << 3) | (uint64_t)o, pos3, mass);
  Node& me = nodes[key];
  double m = 0, cm[3] = {0, 0, 0};
  long cnt = 0;
  for (int o = 0; o < 8; ++o) {
    if (!(me.child & (1u << o))) continue;
    const Node& ch = nodes[(key << 3) | (uint64_t)o];
    m += ch.mass;
    cnt += ch.n;
    for (int a = 0; a < 3; ++a) cm[a] += ch.com[a] * ch.mass;
  }
  div_by(cm, m);
  me.mass = m;
  me.n = cnt;
  std::memcpy(me.com, cm, sizeof(cm));
  std::fill(me.q, me.q + 6, 0.0);
  for (int o = 0; o < 8; ++o) {
    if (!(me.child & (1u << o))) continue;
    const Node& ch = nodes[(key << 3) | (uint64_t)o];
    double x = ch.com[0] - cm[0], y = ch.com[1] - cm[1], z = ch.com[2] - cm[2];
    double mm = ch.mass;
    me.q[1] += 3.0 * mm * (x * y);
    me.q[2] += 3.0 * mm * (x * z);
    me.q[4] += 3.0 * mm * (y * z);
    double xx = x * x, yy = y * y, zz = z * z;
    double d2 = (xx + yy + zz) * mm;
    double m3 = mm * 3.0;
    me.q[0] += m3 * xx - d2;
    me.q[3] += m3 * yy - d2;
    me.q[5] += m3 * zz - d2;
    if (ch.n > 1)
      for (int k = 0; k < 6; ++k) me.q[k] += ch.q[k];
  }
}

// One interaction of ComputeHOTForceInteractionList (src/HashedOctree.hpp:393-459) with the
// softening as a parameter (the reference hard-codes SOFTENING = 0.025, :151).
inline void interact(const double p[3], const double com[3], double m, long n, const double* q, double eps2,
                     double acc[3]) {
  double dx = com[0] - p[0], dy = com[1] - p[1], dz = com[2] - p[2];
  double D2 = dx * dx + dy * dy + dz * dz;
  D2 += eps2;
  double D1 = 1.0 / std::sqrt(D2);
  D2 = 1.0 / D2;
  D1 = D1 * D2;
  acc[0] += m * dx * D1;
  acc[1] += m * dy * D1;
  acc[2] += m * dz * D1;
  if (n > 1 && q) {
    double qx = q[0] * dx + q[1] * dy + q[2] * dz;
    double qy = q[1] * dx + q[3] * dy + q[4] * dz;
    double qz = q[2] * dx + q[4] * dy + q[5] * dz;
    D1 *= D2;
    acc[0] -= qx * D1;
    acc[1] -= qy * D1;
    acc[2] -= qz * D1;
    qx = dx * qx + dy * qy + dz * qz;
    qx *= 2.5;
    D1 *= D2;
    acc[0] += qx * dx * D1;
    acc[1] += qx * dy * D1;
    acc[2] += qx * dz * D1;
  }
}

struct Walker {
  const NodeMap& nodes;
  const double* pos3;
  const double* mass;
  double theta, eps2;
  int mode;
  // Per-body walk of TraverseHOTInteractionList (src/HashedOctree.hpp:336-385) with the MAC
  // of LinearHashedOctree::MAC (src/HashedOctree.cpp:872-885), followed by the list sum.
  // Leaves with one body are self-skipped by exact position (:376); bucket leaves are summed
  // over their members with the same position test.
  struct Item {
    const Node* nd;  // a node (cell, or single-body leaf), or null for a member body of an opened bucket leaf
    int32_t body;
  };
  void body(const double p[3], double acc[3], long* n_cell, long* n_p2p) const {
    std::vector<Item> list;
    gather(p, list);
    acc[0] = acc[1] = acc[2] = 0;
    long nc = 0, np = 0;
    for (const Item& it : list) {
      if (it.nd) {
        interact(p, it.nd->com, it.nd->mass, it.nd->n, mode == 1 ? it.nd->q : nullptr, eps2, acc);
        if (it.nd->n > 1)
          ++nc;
        else
          ++np;
      } else {
        interact(p, pos3 + 3 * it.body, mass[it.body], 1, nullptr, eps2, acc);
        ++np;
      }
    }
    *n_cell = nc;
    *n_p2p = np;
  }
  // The interaction list of the body at p, in the walk's order.
  void gather(const double p[3], std::vector<Item>& list) const {
    std::vector<const Node*> stack;
    list.clear();
    stack.push_back(&nodes.at(1));
    const double th2 = theta * theta;
    while (!stack.empty()) {
      const Node* nd = stack.back();
      stack.pop_back();
      uint64_t key = 0;
      if (nd->child != 0) {
        // the node's key is not stored; children are found through the parent's key
        key = node_key(nd);
        for (int o = 0; o < 8; ++o) {
          if (!(nd->child & (1u << o))) continue;
          const Node* ch = &nodes.at((key << 3) | (uint64_t)o);
          double dx = ch->com[0] - p[0], dy = ch->com[1] - p[1], dz = ch->com[2] - p[2];
          double dist2 = dx * dx + dy * dy + dz * dz;
          double s2 = ch->size * ch->size;
          if ((s2 / dist2) < th2)
            list.push_back({ch, -1});
          else
            stack.push_back(ch);
        }
      } else if (nd->n <= 1 || mode == 0) {
        if (nd->n <= 1) {
          if (nd->com[0] != p[0] || nd->com[1] != p[1] || nd->com[2] != p[2]) list.push_back({nd, -1});
        } else {
          for (uint32_t b : nd->members) {
            const double* q = pos3 + 3 * b;
            if (q[0] != p[0] || q[1] != p[1] || q[2] != p[2]) list.push_back({nullptr, (int32_t)b});
          }
        }
      } else {
        for (uint32_t b : nd->members) {
          const double* q = pos3 + 3 * b;
          if (q[0] != p[0] || q[1] != p[1] || q[2] != p[2]) list.push_back({nullptr, (int32_t)b});
        }
      }
    }
  }
  std::unordered_map<const Node*, uint64_t> keys;
  uint64_t node_key(const Node* nd) const { return keys.at(nd); }
};

}  // namespace

namespace {
void for_threads(size_t n, int nthreads, const std::function<void(size_t, size_t)>& fn) {
  if (nthreads <= 1 || n < 64) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  std::atomic<size_t> next{0};
  const size_t chunk = 256;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&] {
      for (;;) {
        size_t b = next.fetch_add(chunk);
        if (b >= n) break;
        fn(b, std::min(n, b + chunk));
      }
    });
  for (auto& t : th) t.join();
}
}  // namespace

extern "C" {

// OctantBounds(Body*, size_t) (src/OctantUtils.cpp:27-59): centre = sequential FP64 sum of
// positions, then Vec3D::operator/= by N; size = max over bodies and axes of |p_a| - c_a,
// starting from 0.
void orc_bounds(const double* pos3, size_t n, double* c3, double* size) {
  double c[3] = {0, 0, 0};
  for (size_t i = 0; i < n; ++i) {
    c[0] += pos3[3 * i];
    c[1] += pos3[3 * i + 1];
    c[2] += pos3[3 * i + 2];
  }
  div_by(c, (double)n);
  double s = 0;
  for (size_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      double v = std::fabs(pos3[3 * i + a]) - c[a];
      if (v > s) s = v;
    }
  c3[0] = c[0];
  c3[1] = c[1];
  c3[2] = c[2];
  *size = s;
}

// computeMortonKey (src/MortonKeys.hpp:137-181): (p + S) * (2^21 / (2S)), converted with the
// x86-64 double-to-uint64 semantics (x86_trunc_u64), then interleaved with bit 63 set.
void orc_morton_keys(const double* pos3, size_t n, double size, uint64_t* keys) {
  const double frac = (double)(1ull << 21) / (2.0 * size);
  for (size_t i = 0; i < n; ++i) {
    uint64_t w[3];
    for (int a = 0; a < 3; ++a) {
      double s = pos3[3 * i + a] + size;
      s *= frac;
      w[a] = x86_trunc_u64(s);
    }
    keys[i] = (1ull << 63) | (spread_bits(w[0]) << 2) | (spread_bits(w[1]) << 1) | spread_bits(w[2]);
  }
}

// RadixSortBodies permutation (src/Body.hpp:275-302): ThreePassRadixSortMortonKeys
// (src/MortonKeys.hpp:439-470) runs stable counting-sort passes on the byte at shifts
// 0,8,16 / 21,29,37 / 42,50,58 (RadixSortPass :373-411). perm[j] = original index in slot j.
void orc_sort_perm(const uint64_t* keys_in, size_t n, uint32_t* perm) {
  std::vector<uint64_t> k(keys_in, keys_in + n), tk(n);
  std::vector<uint32_t> idx(n), ti(n);
  for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
  const int shifts[9] = {0, 8, 16, 21, 29, 37, 42, 50, 58};
  for (int s : shifts) {
    size_t hist[256] = {0};
    for (size_t i = 0; i < n; ++i) hist[(k[i] >> s) & 0xFF]++;
    size_t off[256];
    off[0] = 0;
    for (int b = 1; b < 256; ++b) off[b] = off[b - 1] + hist[b - 1];
    for (size_t i = 0; i < n; ++i) {
      size_t b = (k[i] >> s) & 0xFF;
      tk[off[b]] = k[i];
      ti[off[b]] = idx[i];
      off[b]++;
    }
    k.swap(tk);
    idx.swap(ti);
  }
  std::memcpy(perm, idx.data(), n * sizeof(uint32_t));
}

// Depth-21 tree path of each body: the root-to-depth-21 descent of insertBody, using the
// octant rule and the child-centre recurrence (src/OctantUtils.hpp:64-101,
// src/HashedNode.cpp:48-70). Node keys are prefixes: key >> 3*(21-d) at depth d.
void orc_tree_keys(const double* pos3, size_t n, const double* c3, double edge, uint64_t* tkeys) {
  for (size_t i = 0; i < n; ++i) {
    double c[3] = {c3[0], c3[1], c3[2]}, s = edge;
    uint64_t key = 1;
    for (int d = 0; d < kMaxDepth; ++d) {
      int o = octant_of(c, pos3 + 3 * i);
      key = (key << 3) | (uint64_t)o;
      double cc[3], cs;
      child_bounds(c, s, o, cc, &cs);
      c[0] = cc[0];
      c[1] = cc[1];
      c[2] = cc[2];
      s = cs;
    }
    tkeys[i] = key;
  }
}

// Guard: number of depth-21 cells holding more than one body. The reference (leaf capacity 1)
// overflows its node key on such inputs (src/HashedOctree.cpp:162-170), so its oracle runs
// only when this is 0.
long orc_guard(const double* pos3, size_t n, const double* c3, double edge) {
  std::vector<uint64_t> k(n);
  orc_tree_keys(pos3, n, c3, edge, k.data());
  std::sort(k.begin(), k.end());
  long dup = 0;
  for (size_t i = 1; i < n; ++i) dup += (k[i] == k[i - 1] && (i < 2 || k[i - 1] != k[i - 2]));
  return dup;
}

// Tree build (insertion in the given body order, which is the sorted order in the reference)
// plus the multipole pass of the chosen mode. Output sorted by node key. Returns the node
// count, or -1 if cap is too small.
long orc_build(const double* pos3, const double* mass, size_t n, const double* c3, double edge, int L, int mode,
               size_t cap, uint64_t* keys, int64_t* counts, double* masses, double* com3, uint8_t* childbyte,
               double* quad6) {
  NodeMap nodes;
  insert_all(nodes, pos3, mass, n, c3, edge, L < 1 ? 1 : L);
  if (mode == 1 && n > 0) upsweep(nodes, 1, pos3, mass);
  std::vector<uint64_t> order;
  order.reserve(nodes.size());
  for (auto& kv : nodes) order.push_back(kv.first);
  std::sort(order.begin(), order.end());
  if (order.size() > cap) return -1;
  for (size_t j = 0; j < order.size(); ++j) {
    const Node& nd = nodes[order[j]];
    keys[j] = order[j];
    if (counts) counts[j] = nd.n;
    if (masses) masses[j] = nd.mass;
    if (com3)
      for (int a = 0; a < 3; ++a) com3[3 * j + a] = nd.com[a];
    if (childbyte) childbyte[j] = nd.child;
    if (quad6)
      for (int k = 0; k < 6; ++k) quad6[6 * j + k] = nd.q[k];
  }
  return (long)order.size();
}

// Tree build + ComputeHOTOctreeForce-equivalent walk for the bodies listed in targets (all
// bodies when targets is null). acc3 is written (not accumulated), per target.
int orc_force(const double* pos3, const double* mass, size_t n, const double* c3, double edge, int L, int mode,
              double theta, double eps, const uint32_t* targets, size_t nt, int nthreads, double* acc3,
              int64_t* n_cell, int64_t* n_p2p) {
  if (n == 0) return 0;
  NodeMap nodes;
  insert_all(nodes, pos3, mass, n, c3, edge, L < 1 ? 1 : L);
  if (mode == 1) upsweep(nodes, 1, pos3, mass);
  Walker w{nodes, pos3, mass, theta, eps * eps, mode, {}};
  w.keys.reserve(nodes.size());
  for (auto& kv : nodes) w.keys[&kv.second] = kv.first;
  size_t cnt = targets ? nt : n;
  for_threads(cnt, nthreads, [&](size_t b, size_t e) {
    for (size_t t = b; t < e; ++t) {
      size_t i = targets ? targets[t] : t;
      long nc, np;
      w.body(pos3 + 3 * i, acc3 + 3 * t, &nc, &np);
      if (n_cell) n_cell[t] = nc;
      if (n_p2p) n_p2p[t] = np;
    }
  });
  return 0;
}

// FP64 O(N^2) direct sum with Plummer softening, G = 1, for the listed targets: acceleration
// and potential (-sum m_j / sqrt(d^2 + eps^2), j != i).
void orc_direct(const double* pos3, const double* mass, size_t n, const uint32_t* targets, size_t nt, double eps,
                int nthreads, double* acc3, double* pot) {
  const double e2 = eps * eps;
  for_threads(nt, nthreads, [&](size_t b, size_t e) {
    for (size_t t = b; t < e; ++t) {
      size_t i = targets ? targets[t] : t;
      const double* p = pos3 + 3 * i;
      double ax = 0, ay = 0, az = 0, ph = 0;
      for (size_t j = 0; j < n; ++j) {
        if (j == i) continue;
        double dx = pos3[3 * j] - p[0], dy = pos3[3 * j + 1] - p[1], dz = pos3[3 * j + 2] - p[2];
        double r2 = dx * dx + dy * dy + dz * dz + e2;
        double ri = 1.0 / std::sqrt(r2);
        double f = mass[j] * ri * ri * ri;
        ax += f * dx;
        ay += f * dy;
        az += f * dz;
        ph -= mass[j] * ri;
      }
      acc3[3 * t] = ax;
      acc3[3 * t + 1] = ay;
      acc3[3 * t + 2] = az;
      if (pot) pot[t] = ph;
    }
  });
}

// Kick + drift (ComputePositionAtHalfTimeStep, src/Body.hpp:306-313) and kick
// (ComputeVelocityAndPosition, :317-324).
void orc_kick_drift(double* pos3, double* vel3, const double* acc3, size_t n, double dt) {
  for (size_t i = 0; i < 3 * n; ++i) {
    vel3[i] += acc3[i] * dt * 0.5;
    pos3[i] += vel3[i] * dt;
  }
}
void orc_kick(double* vel3, const double* acc3, size_t n, double dt) {
  for (size_t i = 0; i < 3 * n; ++i) vel3[i] += acc3[i] * dt * 0.5;
}

// nsteps of the per-frame sequence of ofApp::update + draw (src/ofApp.cpp:169-177, 248-282):
// bounds(x_n) -> Morton keys(x_n) -> sort -> kick+drift -> build on x_{n+1} with the bounds of
// x_n (root edge = S * edge_factor) -> force -> kick. State arrays are reordered in place by
// the sort. acc_follows_body = 0 keeps the reference's behaviour of not reordering the
// acceleration array in the sort (RadixSortBodies touches only the Body array); 1 reorders it
// with the bodies. stage_s (optional, 6 doubles) accumulates seconds per stage: bounds+keys,
// sort, kick+drift, build, force, kick. perm_out (optional) receives slot -> original index.
int orc_steps(double* pos3, double* vel3, double* mass, double* acc3, size_t n, double dt, double theta,
              double eps, double edge_factor, int L, int mode, int nsteps, int acc_follows_body, int nthreads,
              double* stage_s, uint32_t* perm_out) {
  auto now = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
  std::vector<uint32_t> composed(n);
  for (size_t i = 0; i < n; ++i) composed[i] = (uint32_t)i;
  std::vector<uint64_t> keys(n);
  std::vector<uint32_t> perm(n);
  std::vector<double> tp(3 * n), tv(3 * n), ta(3 * n), tm(n);
  std::vector<uint32_t> tc(n);
  for (int s = 0; s < nsteps; ++s) {
    double t0 = now();
    double c[3], S;
    orc_bounds(pos3, n, c, &S);
    orc_morton_keys(pos3, n, S, keys.data());
    double t1 = now();
    orc_sort_perm(keys.data(), n, perm.data());
    for (size_t j = 0; j < n; ++j) {
      size_t i = perm[j];
      for (int a = 0; a < 3; ++a) {
        tp[3 * j + a] = pos3[3 * i + a];
        tv[3 * j + a] = vel3[3 * i + a];
        ta[3 * j + a] = acc_follows_body ? acc3[3 * i + a] : acc3[3 * j + a];
      }
      tm[j] = mass[i];
      tc[j] = composed[i];
    }
    std::memcpy(pos3, tp.data(), 3 * n * sizeof(double));
    std::memcpy(vel3, tv.data(), 3 * n * sizeof(double));
    std::memcpy(acc3, ta.data(), 3 * n * sizeof(double));
    std::memcpy(mass, tm.data(), n * sizeof(double));
    std::memcpy(composed.data(), tc.data(), n * sizeof(uint32_t));
    double t2 = now();
    orc_kick_drift(pos3, vel3, acc3, n, dt);
    double t3 = now();
    // build + force: orc_force builds the tree internally; its build time is measured by a
    // separate build so the stage split stays visible
    NodeMap nodes;
    insert_all(nodes, pos3, mass, n, c, S * edge_factor, L < 1 ? 1 : L);
    if (mode == 1 && n > 0) upsweep(nodes, 1, pos3, mass);
    double t4 = now();
    if (n > 0) {
      Walker w{nodes, pos3, mass, theta, eps * eps, mode, {}};
      w.keys.reserve(nodes.size());
      for (auto& kv : nodes) w.keys[&kv.second] = kv.first;
      for_threads(n, nthreads, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
          long nc, np;
          w.body(pos3 + 3 * i, acc3 + 3 * i, &nc, &np);
        }
      });
    }
    double t5 = now();
    orc_kick(vel3, acc3, n, dt);
    double t6 = now();
    if (stage_s) {
      stage_s[0] += t1 - t0;
      stage_s[1] += t2 - t1;
      stage_s[2] += t3 - t2;
      stage_s[3] += t4 - t3;
      stage_s[4] += t5 - t4;
      stage_s[5] += t6 - t5;
    }
  }
  if (perm_out) std::memcpy(perm_out, composed.data(), n * sizeof(uint32_t));
  return 0;
}

// Timing helper for the CPU baseline: build the tree once over all n bodies, then walk only
// the listed targets, returning seconds for build and walk separately.
int orc_time_sample(const double* pos3, const double* mass, size_t n, const double* c3, double edge, int L, int mode,
                    double theta, double eps, const uint32_t* targets, size_t nt, int nthreads, double* build_s,
                    double* walk_s, double* acc3) {
  auto now = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
  double t0 = now();
  NodeMap nodes;
  insert_all(nodes, pos3, mass, n, c3, edge, L < 1 ? 1 : L);
  if (mode == 1 && n > 0) upsweep(nodes, 1, pos3, mass);
  double t1 = now();
  Walker w{nodes, pos3, mass, theta, eps * eps, mode, {}};
  w.keys.reserve(nodes.size());
  for (auto& kv : nodes) w.keys[&kv.second] = kv.first;
  double t1b = now();
  for_threads(nt, nthreads, [&](size_t b, size_t e) {
    for (size_t t = b; t < e; ++t) {
      long nc, np;
      w.body(pos3 + 3 * targets[t], acc3 + 3 * t, &nc, &np);
    }
  });
  double t2 = now();
  *build_s = (t1 - t0) + (t1b - t1);
  *walk_s = t2 - t1b;
  return 0;
}

}  // extern "C"

// ---- Differentiable trajectory (checker for bh_adjoint_forward / bh_step_backward) ----
// The reference has no reverse mode; these follow the library's differentiable path: bodies keep
// their order, a(x_0) comes from a tree over x_0 with the bounds of x_0, step n builds its tree
// over x_{n+1} with the bounds of x_n (root edge = S * edge_factor), quadrupole multipoles, and
// the interaction lists of the forward pass are held fixed.
namespace {

// Interaction lists of one force evaluation, held fixed for replays.
struct FrozenForce {
  std::vector<uint32_t> cell_off{0};  // cell c: member bodies cell_mem[cell_off[c] .. cell_off[c + 1])
  std::vector<uint32_t> cell_mem;
  std::vector<uint32_t> off;          // body i: entries ent[off[i] .. off[i + 1])
  std::vector<int32_t> ent;           // >= 0: point source body; < 0: cell -(c + 1)
};

struct Frozen {
  size_t n = 0;
  double dt = 0, eps = 0;
  int nsteps = 0;
  std::vector<FrozenForce> f;  // a(x_0), a(x_1), ..., a(x_nsteps)
};

void collect_members(const NodeMap& nodes, uint64_t key, std::vector<uint32_t>& out) {
  const Node& nd = nodes.at(key);
  if (nd.child == 0) {
    out.insert(out.end(), nd.members.begin(), nd.members.end());
    return;
  }
  for (int o = 0; o < 8; ++o)
    if (nd.child & (1u << o)) collect_members(nodes, (key << 3) | (uint64_t)o, out);
}

// Tree over pos (root centre c, edge), quadrupole upsweep, every body's interaction list.
void record_force(const double* pos3, const double* mass, size_t n, const double c[3], double edge, int L,
                  double theta, double eps, int nthreads, FrozenForce& ff) {
  NodeMap nodes;
  insert_all(nodes, pos3, mass, n, c, edge, L < 1 ? 1 : L);
  upsweep(nodes, 1, pos3, mass);
  Walker w{nodes, pos3, mass, theta, eps * eps, 1, {}};
  w.keys.reserve(nodes.size());
  for (auto& kv : nodes) w.keys[&kv.second] = kv.first;
  std::vector<std::vector<Walker::Item>> lists(n);
  for_threads(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) w.gather(pos3 + 3 * i, lists[i]);
  });
  std::unordered_map<const Node*, int32_t> cell_id;
  ff = FrozenForce();
  ff.off.assign(n + 1, 0);
  for (size_t i = 0; i < n; ++i) {
    ff.off[i] = (uint32_t)ff.ent.size();
    for (const Walker::Item& it : lists[i]) {
      if (!it.nd) {
        ff.ent.push_back(it.body);
      } else if (it.nd->n <= 1) {
        ff.ent.push_back((int32_t)it.nd->members[0]);  // single-body leaf
      } else {
        auto f = cell_id.find(it.nd);
        int32_t id;
        if (f == cell_id.end()) {
          id = (int32_t)cell_id.size();
          cell_id.emplace(it.nd, id);
          collect_members(nodes, w.node_key(it.nd), ff.cell_mem);
          ff.cell_off.push_back((uint32_t)ff.cell_mem.size());
        } else {
          id = f->second;
        }
        ff.ent.push_back(-(id + 1));
      }
    }
  }
  ff.off[n] = (uint32_t)ff.ent.size();
}

// Accelerations from frozen lists: each cell's mass, centre of mass and quadrupole are
// recomputed from its members' current positions.
void frozen_force(const FrozenForce& ff, const double* pos3, const double* mass, size_t n, double eps2,
                  int nthreads, double* acc3) {
  const size_t nc = ff.cell_off.size() - 1;
  std::vector<double> cm(4 * nc), cq(6 * nc);
  for_threads(nc, nthreads, [&](size_t b, size_t e) {
    for (size_t c = b; c < e; ++c) {
      double m = 0, x[3] = {0, 0, 0};
      for (uint32_t k = ff.cell_off[c]; k < ff.cell_off[c + 1]; ++k) {
        const uint32_t j = ff.cell_mem[k];
        m += mass[j];
        for (int a = 0; a < 3; ++a) x[a] += mass[j] * pos3[3 * j + a];
      }
      for (int a = 0; a < 3; ++a) x[a] /= m;
      double q[6] = {0, 0, 0, 0, 0, 0};
      for (uint32_t k = ff.cell_off[c]; k < ff.cell_off[c + 1]; ++k) {
        const uint32_t j = ff.cell_mem[k];
        const double rx = pos3[3 * j] - x[0], ry = pos3[3 * j + 1] - x[1], rz = pos3[3 * j + 2] - x[2];
        const double mj = mass[j], r2 = rx * rx + ry * ry + rz * rz;
        q[0] += mj * (3 * rx * rx - r2);
        q[1] += mj * 3 * rx * ry;
        q[2] += mj * 3 * rx * rz;
        q[3] += mj * (3 * ry * ry - r2);
        q[4] += mj * 3 * ry * rz;
        q[5] += mj * (3 * rz * rz - r2);
      }
      cm[4 * c] = x[0];
      cm[4 * c + 1] = x[1];
      cm[4 * c + 2] = x[2];
      cm[4 * c + 3] = m;
      for (int k = 0; k < 6; ++k) cq[6 * c + k] = q[k];
    }
  });
  for_threads(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      double a[3] = {0, 0, 0};
      for (uint32_t k = ff.off[i]; k < ff.off[i + 1]; ++k) {
        const int32_t t = ff.ent[k];
        if (t >= 0) {
          interact(pos3 + 3 * i, pos3 + 3 * t, mass[t], 1, nullptr, eps2, a);
        } else {
          const size_t c = (size_t)(-t - 1);
          interact(pos3 + 3 * i, &cm[4 * c], cm[4 * c + 3], 2, &cq[6 * c], eps2, a);
        }
      }
      acc3[3 * i] = a[0];
      acc3[3 * i + 1] = a[1];
      acc3[3 * i + 2] = a[2];
    }
  });
}

// KDK trajectory in place on (x, v); records the lists first when `record`.
void frozen_traj(Frozen& fr, bool record, double* x, double* v, const double* m, double theta, double edge_factor,
                 int L, int nthreads) {
  const size_t n = fr.n;
  const double dt = fr.dt, eps2 = fr.eps * fr.eps;
  std::vector<double> a(3 * n);
  double c[3], S;
  if (record) {
    fr.f.assign(fr.nsteps + 1, FrozenForce());
    orc_bounds(x, n, c, &S);
    record_force(x, m, n, c, S * edge_factor, L, theta, fr.eps, nthreads, fr.f[0]);
  }
  frozen_force(fr.f[0], x, m, n, eps2, nthreads, a.data());
  for (int s = 0; s < fr.nsteps; ++s) {
    if (record) orc_bounds(x, n, c, &S);
    orc_kick_drift(x, v, a.data(), n, dt);
    if (record) record_force(x, m, n, c, S * edge_factor, L, theta, fr.eps, nthreads, fr.f[s + 1]);
    frozen_force(fr.f[s + 1], x, m, n, eps2, nthreads, a.data());
    orc_kick(v, a.data(), n, dt);
  }
}

// (xb, mb) += vector-Jacobian product of the FP64 direct-sum acceleration at x applied to ab.
void direct_vjp(const double* x, const double* m, size_t n, double eps2, const double* ab, int nthreads, double* xb,
                double* mb) {
  for_threads(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      double gx = 0, gy = 0, gz = 0, gm = 0;
      const double* ai = ab + 3 * i;
      for (size_t j = 0; j < n; ++j) {
        if (j == i) continue;
        const double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1], dz = x[3 * j + 2] - x[3 * i + 2];
        const double r2 = dx * dx + dy * dy + dz * dz + eps2;
        const double ri = 1.0 / std::sqrt(r2);
        const double w3 = ri * ri * ri, w5 = w3 * ri * ri;
        // a_i's dependence on x_i (through d = x_j - x_i)
        const double adi = ai[0] * dx + ai[1] * dy + ai[2] * dz;
        gx -= m[j] * (w3 * ai[0] - 3 * w5 * adi * dx);
        gy -= m[j] * (w3 * ai[1] - 3 * w5 * adi * dy);
        gz -= m[j] * (w3 * ai[2] - 3 * w5 * adi * dz);
        // a_j's dependence on x_i and m_i (source i, d' = x_i - x_j = -d)
        const double* aj = ab + 3 * j;
        const double adj = -(aj[0] * dx + aj[1] * dy + aj[2] * dz);
        gx += m[i] * (w3 * aj[0] + 3 * w5 * adj * dx);
        gy += m[i] * (w3 * aj[1] + 3 * w5 * adj * dy);
        gz += m[i] * (w3 * aj[2] + 3 * w5 * adj * dz);
        gm += w3 * adj;
      }
      xb[3 * i] += gx;
      xb[3 * i + 1] += gy;
      xb[3 * i + 2] += gz;
      mb[i] += gm;
    }
  });
}

}  // namespace

extern "C" {

// Records a trajectory with its interaction lists (returns a handle; pos_out / vel_out get the
// final state).
void* orc_frozen_record(const double* pos3, const double* vel3, const double* mass, size_t n, double dt,
                        double theta, double eps, double edge_factor, int L, int nsteps, int nthreads,
                        double* pos_out, double* vel_out) {
  Frozen* fr = new Frozen();
  fr->n = n;
  fr->dt = dt;
  fr->eps = eps;
  fr->nsteps = nsteps;
  std::memcpy(pos_out, pos3, 3 * n * sizeof(double));
  std::memcpy(vel_out, vel3, 3 * n * sizeof(double));
  frozen_traj(*fr, true, pos_out, vel_out, mass, theta, edge_factor, L, nthreads);
  return fr;
}

// Re-runs the recorded trajectory's map (lists held fixed) from another initial state.
void orc_frozen_run(void* h, const double* pos3, const double* vel3, const double* mass, int nthreads,
                    double* pos_out, double* vel_out) {
  Frozen* fr = (Frozen*)h;
  std::memcpy(pos_out, pos3, 3 * fr->n * sizeof(double));
  std::memcpy(vel_out, vel3, 3 * fr->n * sizeof(double));
  frozen_traj(*fr, false, pos_out, vel_out, mass, 0, 1, 1, nthreads);
}

// Total list entries over all recorded force evaluations (cells and points).
long orc_frozen_entries(void* h) {
  long t = 0;
  for (const FrozenForce& f : ((Frozen*)h)->f) t += (long)f.ent.size();
  return t;
}

void orc_frozen_free(void* h) { delete (Frozen*)h; }

// FP64 direct-sum KDK trajectory and its adjoint: gradients with respect to the initial
// positions, velocities and masses of a loss whose gradients with respect to the final
// positions and velocities are dl_dx / dl_dv.
void orc_direct_adjoint(const double* pos3, const double* vel3, const double* mass, size_t n, double dt, double eps,
                        int nsteps, const double* dl_dx, const double* dl_dv, int nthreads, double* pos_out,
                        double* vel_out, double* gx, double* gv, double* gm) {
  const double e2 = eps * eps, h = 0.5 * dt;
  std::vector<double> xs(3 * n * (size_t)(nsteps + 1)), v(vel3, vel3 + 3 * n), a(3 * n);
  std::memcpy(xs.data(), pos3, 3 * n * sizeof(double));
  orc_direct(xs.data(), mass, n, nullptr, n, eps, nthreads, a.data(), nullptr);
  for (int s = 0; s < nsteps; ++s) {
    double* x = xs.data() + 3 * n * (size_t)(s + 1);
    std::memcpy(x, x - 3 * n, 3 * n * sizeof(double));
    orc_kick_drift(x, v.data(), a.data(), n, dt);
    orc_direct(x, mass, n, nullptr, n, eps, nthreads, a.data(), nullptr);
    orc_kick(v.data(), a.data(), n, dt);
  }
  std::memcpy(pos_out, xs.data() + 3 * n * (size_t)nsteps, 3 * n * sizeof(double));
  std::memcpy(vel_out, v.data(), 3 * n * sizeof(double));
  std::vector<double> xb(3 * n, 0.0), vb(3 * n, 0.0), carry(3 * n, 0.0), ab(3 * n), mb(n, 0.0);
  if (dl_dx) std::memcpy(xb.data(), dl_dx, 3 * n * sizeof(double));
  if (dl_dv) std::memcpy(vb.data(), dl_dv, 3 * n * sizeof(double));
  for (int s = nsteps - 1; s >= 0; --s) {
    for (size_t k = 0; k < 3 * n; ++k) ab[k] = h * vb[k] + carry[k];
    direct_vjp(xs.data() + 3 * n * (size_t)(s + 1), mass, n, e2, ab.data(), nthreads, xb.data(), mb.data());
    for (size_t k = 0; k < 3 * n; ++k) {
      vb[k] += dt * xb[k];
      carry[k] = h * vb[k];
    }
  }
  direct_vjp(xs.data(), mass, n, e2, carry.data(), nthreads, xb.data(), mb.data());
  std::memcpy(gx, xb.data(), 3 * n * sizeof(double));
  std::memcpy(gv, vb.data(), 3 * n * sizeof(double));
  std::memcpy(gm, mb.data(), n * sizeof(double));
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// The reference app's solar-system scene (SetupSolarSystem, src/PhysicsHelpers.hpp:268-683),
// restated in FP64 with the same random draws as the library's device generator.
// ---------------------------------------------------------------------------------------
namespace {

// The library's counter-based uniform in (0, 1): splitmix64's output mix of (seed, body, draw).
uint64_t scene_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double scene_uniform(uint64_t seed, uint64_t body, uint32_t draw) {
  const uint64_t z = scene_mix(scene_mix(seed + 0x9e3779b97f4a7c15ull * (body + 1)) ^ (0x632be59bd9b4e019ull * (draw + 1)));
  return ((double)(z >> 11) + 0.5) * 0x1p-53;
}
// ofRandom(lo, hi) as a float: lo + (hi - lo) u, u the uniform rounded to float.
float scene_draw(uint64_t seed, uint64_t body, uint32_t k, float lo, float hi) {
  const float u = (float)scene_uniform(seed, body, k);
  return lo + (hi - lo) * u;
}

const double kSceneG = 6.67430e-11, kSceneSun = 1.989e30, kSceneAU = 149597870700.0;
const double kSceneDeg = 0.01745329252;  // toRadians, src/PhysicsHelpers.hpp:701-708

// Newton from E = M until |step| <= 1e-10 (at most 100 steps), then the true anomaly and
// calculatePositionAndVelocity (src/PhysicsHelpers.hpp:729-790).
void scene_true_anomaly(double e, double a, double i, double node, double w, double M, double mu, double x[3],
                        double v[3]) {
  double E = M, delta;
  int iter = 0;
  do {
    double f = E - e * std::sin(E) - M;
    double fp = 1 - e * std::cos(E);
    delta = -f / fp;
    E += delta;
    iter++;
  } while (std::fabs(delta) > 1e-10 && iter < 100);
  double nu = 2 * std::atan2(std::sqrt(1 + e) * std::sin(E / 2), std::sqrt(1 - e) * std::cos(E / 2));
  double r = a * (1 - e * std::cos(E));
  double xo = r * std::cos(nu), yo = r * std::sin(nu);
  double cn = std::cos(node), sn = std::sin(node), cw = std::cos(w), sw = std::sin(w), ci = std::cos(i),
         si = std::sin(i);
  x[0] = xo * (cn * cw - sn * sw * ci) - yo * (cn * sw + sn * cw * ci);
  x[1] = xo * (sn * cw + cn * sw * ci) + yo * (cn * cw * ci - sn * sw);
  x[2] = xo * (sw * si) + yo * (cw * si);
  double h = std::sqrt(mu * a * (1 - e * e));
  double vxo = -mu / h * std::sin(nu), vyo = mu / h * (e + std::cos(nu));
  v[0] = vxo * (cn * cw - sn * sw * ci) - vyo * (cn * sw + sn * cw * ci);
  v[1] = vxo * (sn * cw + cn * sw * ci) + vyo * (cn * cw * ci - sn * sw);
  v[2] = vxo * (sw * si) + vyo * (cw * si);
}

// computeCartesianFromOrbital (src/SolarSystem.h:33-108): 100 Newton steps, perifocal state,
// rotation.
void scene_eccentric(double a, double e, double i, double node, double w, double M, double mu, double x[3],
                     double v[3]) {
  double E = M;
  for (int it = 0; it < 100; it++) {
    double f = E - e * std::sin(E) - M;
    double fp = 1.0 - e * std::cos(E);
    E = E - f / fp;
  }
  double cE = std::cos(E), sE = std::sin(E), s1 = std::sqrt(1.0 - e * e);
  double xp = a * (cE - e), yp = a * s1 * sE;
  double n = std::sqrt(mu / (a * a * a));
  double edot = n / (1.0 - e * cE);
  double vxp = -a * edot * sE, vyp = a * edot * s1 * cE;
  double cn = std::cos(node), sn = std::sin(node), ci = std::cos(i), si = std::sin(i), cw = std::cos(w),
         sw = std::sin(w);
  x[0] = (cn * cw - sn * sw * ci) * xp + (-cn * sw - sn * cw * ci) * yp;
  x[1] = (sn * cw + cn * sw * ci) * xp + (-sn * sw + cn * cw * ci) * yp;
  x[2] = (sw * si) * xp + (cw * si) * yp;
  v[0] = (cn * cw - sn * sw * ci) * vxp + (-cn * sw - sn * cw * ci) * vyp;
  v[1] = (sn * cw + cn * sw * ci) * vxp + (-sn * sw + cn * cw * ci) * vyp;
  v[2] = (sw * si) * vxp + (cw * si) * vyp;
}

}  // namespace

extern "C" {

// Scene of n bodies: out7[7 i ..] = x, y, z, vx, vy, vz, m in SI units (FP64, before any
// rounding to the library's FP32 state).
void orc_solar_system(uint64_t seed, size_t n, double* out7) {
  // planet table of the scene (src/PhysicsHelpers.hpp:298-397): e, a (AU), i, node, periapsis
  // (degrees), mean anomaly (used as radians), mass (kg, also used as mu)
  static const double planets[8][7] = {
      {0.205630, 0.387098, 7.00487, 48.331, 29.124, 174.795, 3.3011e23},
      {0.006772, 0.723332, 3.39471, 76.6807, 54.8523, 50.416, 4.8675e24},
      {0.016711, 1.000000, 0.00005, 348.73936, 114.20783, 357.51716, 5.97237e24},
      {0.093394, 1.523679, 1.85061, 49.57854, 286.502, 19.3564, 6.4171e23},
      {0.0489, 5.2026, 1.304, 100.464, 273.867, 20.02, 1.8982e27},
      {0.0565, 9.5549, 2.485, 113.665, 339.392, 317.02, 5.6834e26},
      {0.046381, 19.2184, 0.773, 74.006, 96.998857, 142.2386, 8.6810e25},
      {0.008678, 30.1104, 1.767, 131.784, 273.187, 48.12369, 1.02413e26},
  };
  auto planet = [&](int p, double x[3], double v[3]) {
    const double* q = planets[p];
    scene_true_anomaly(q[0], q[1] * kSceneAU, q[2] * kSceneDeg, q[3] * kSceneDeg, q[4] * kSceneDeg, q[5], q[6], x,
                       v);
  };
  for (size_t i = 0; i < n; ++i) {
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, m = 0;
    if (i == 0) {
      m = kSceneSun;
    } else if (i <= 8) {
      planet((int)i - 1, x, v);
      m = planets[i - 1][6];
    } else if (i == 9) {
      double xe[3], ve[3];
      planet(2, xe, ve);
      scene_true_anomaly(0.0549, 3.844e8, 5.145 * kSceneDeg, 125.08 * kSceneDeg, 318.15 * kSceneDeg, 135.27,
                         kSceneG * 5.97237e24, x, v);
      for (int k = 0; k < 3; ++k) {
        x[k] += xe[k] * 1.1;
        v[k] += ve[k];
      }
      m = 7.34767309e22;
    } else {
      const bool belt = (double)i < (double)n * 0.5;
      const float e = belt ? scene_draw(seed, i, 0, 0.0f, 0.2f) : scene_draw(seed, i, 0, 0.8f, 0.99f);
      const float a = belt ? scene_draw(seed, i, 1, 2.2f, 3.2f) : scene_draw(seed, i, 1, 1000.0f, 100000.0f);
      const float inc = belt ? scene_draw(seed, i, 2, 0.0f, 15.0f) : scene_draw(seed, i, 2, 0.0f, 180.0f);
      const float node = scene_draw(seed, i, 3, 0.0f, 360.0f);
      const float w = scene_draw(seed, i, 4, 0.0f, 360.0f);
      const float M = scene_draw(seed, i, 5, 0.0f, 360.0f);
      const float mm = belt ? scene_draw(seed, i, 6, 1e15f, 1e21f) : scene_draw(seed, i, 6, 1e12f, 1e17f);
      scene_eccentric((double)a * kSceneAU, e, inc * kSceneDeg, node * kSceneDeg, w * kSceneDeg, M * kSceneDeg,
                      kSceneG * kSceneSun, x, v);
      m = mm;
    }
    double* o = out7 + 7 * i;
    for (int k = 0; k < 3; ++k) {
      o[k] = x[k];
      o[3 + k] = v[k];
    }
    o[6] = m;
  }
}

}  // extern "C"

extern "C" {

// decodeMortonKey (src/MortonKeys.hpp:204-228): the 21 bits of each axis de-interleaved from the
// key (x from bits 3i + 2, y from 3i + 1, z from 3i), then x_int / 2^21 * 2 * size - size.
void orc_decode_morton(const uint64_t* keys, size_t n, double size, double* pos3) {
  for (size_t i = 0; i < n; ++i) {
    uint64_t q[3] = {0, 0, 0};
    for (int b = 0; b < 21; ++b)
      for (int a = 0; a < 3; ++a) q[a] |= ((keys[i] >> (3 * b + 2 - a)) & 1ull) << b;
    for (int a = 0; a < 3; ++a) pos3[3 * i + a] = (double)q[a] / 2097152.0 * 2.0 * size - size;
  }
}

}  // extern "C"
