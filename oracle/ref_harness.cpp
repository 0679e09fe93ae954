// REF-LITERAL harness: a C ABI around the reference's own, unmodified hot-path code.
//
// TEST INFRASTRUCTURE ONLY (the oracle). Only tests/, the golden-fixture script and
// bench.py's CPU-baseline leg load this library, and only as a checker / baseline.
//
// This file contains no reference code. It is compiled together with the reference's
// translation units src/{MathUtils,Body,OctantUtils,HashedNode,HashedOctree}.cpp, read
// in place from the reference checkout by oracle/build_oracle.py, and a headless
// ofMain.h (oracle/ref_shim/ofMain.h). The output goes to oracle/_ref/ (git-ignored).
//
// Entry points and the reference code each one drives:
//   ref_bounds        OctantBounds::OctantBounds(Body*, size_t)        src/OctantUtils.cpp:27-59
//   ref_morton_keys   computeMortonKey                                 src/MortonKeys.hpp:137-181
//   ref_decode_morton decodeMortonKey                                  src/MortonKeys.hpp:204-228
//   ref_sort_bodies   RadixSortBodies                                  src/Body.hpp:275-302
//   ref_guard         DetermineOctant / GetChildKey / HOTNode child ctor src/OctantUtils.hpp:64-101,
//                                                                      src/HashedNode.cpp:48-70
//   ref_build_nodes   buildLinearHashedOctreeInPlace                   src/HashedOctree.hpp:211-244
//   ref_force         ComputeHOTOctreeForce                            src/HashedOctree.hpp:262-273
//   ref_app_steps     the per-frame sequence of ofApp::update + draw   src/ofApp.cpp:169-177, 248-282
//
// The reference's insertion overflows its 64-bit node key (and then frees a live node,
// src/HashedOctree.cpp:162-170) whenever two bodies share a depth-21 cell. Every entry
// point that builds a tree runs ref_guard first and refuses such inputs (returns -2).
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <vector>

#include "HashedOctree.hpp"

namespace {

Body* make_bodies(const double* pos3, const double* vel3, const double* mass, size_t n) {
  Body* b = new Body[n];
  for (size_t i = 0; i < n; ++i) {
    Vec3D p(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]);
    Vec3D v = vel3 ? Vec3D(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2]) : Vec3D(0.0, 0.0, 0.0);
    b[i] = Body(p, v, mass ? mass[i] : 1.0);
    b[i].displayRadius = (double)i;  // tag: the original index travels with the body
  }
  return b;
}

// Depth-21 tree path of one body, using the reference's own octant and child-centre code.
spatialKey depth21_key(const Vec3D& pos, const OctantBounds& root) {
  HOTNode node(root, ROOT_KEY);
  Vec3D p = pos;
  for (int d = 0; d < 21; ++d) {
    OctantEnum o = DetermineOctant(node.nodeBounds.center, p);
    HOTNode child(&node, o, p, 1.0);
    node = child;
  }
  return node.nodeKey;
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

int ref_bounds(const double* pos3, size_t n, double* center3, double* size) {
  Body* b = make_bodies(pos3, nullptr, nullptr, n);
  OctantBounds ob(b, n);
  center3[0] = ob.center.x;
  center3[1] = ob.center.y;
  center3[2] = ob.center.z;
  *size = ob.size;
  delete[] b;
  return 0;
}

int ref_morton_keys(const double* pos3, size_t n, double size, uint64_t* keys) {
  for (size_t i = 0; i < n; ++i) {
    Vec3D p(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]);
    keys[i] = computeMortonKey(p, size);
  }
  return 0;
}

int ref_decode_morton(const uint64_t* keys, size_t n, double size, double* pos3) {
  for (size_t i = 0; i < n; ++i) {
    const Vec3D p = decodeMortonKey(keys[i], size);
    pos3[3 * i] = p.x;
    pos3[3 * i + 1] = p.y;
    pos3[3 * i + 2] = p.z;
  }
  return 0;
}

// Permutation applied by RadixSortBodies: perm[j] = original index of the body in slot j.
int ref_sort_bodies(const uint64_t* keys, size_t n, uint32_t* perm) {
  Body* b = make_bodies(std::vector<double>(3 * n, 0.0).data(), nullptr, nullptr, n);
  for (size_t i = 0; i < n; ++i) b[i].bodyKey = keys[i];
  RadixSortBodies(b, n);
  for (size_t j = 0; j < n; ++j) perm[j] = (uint32_t)b[j].displayRadius;
  delete[] b;
  return 0;
}

// Number of depth-21 cells holding more than one body (0 = the reference can build it).
long ref_guard(const double* pos3, size_t n, const double* center3, double edge) {
  OctantBounds root(Vec3D(center3[0], center3[1], center3[2]), edge);
  std::vector<spatialKey> k(n);
  for (size_t i = 0; i < n; ++i) k[i] = depth21_key(Vec3D(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]), root);
  std::sort(k.begin(), k.end());
  long dup = 0;
  for (size_t i = 1; i < n; ++i) dup += (k[i] == k[i - 1] && (i < 2 || k[i - 1] != k[i - 2]));
  return dup;
}

// Builds the reference tree over the bodies in the given (insertion) order and dumps it, in
// key order. box4 (optional) receives each node's nodeBounds as (centre x, y, z, size): the
// cube the reference's child constructor gives it (src/HashedNode.cpp:48-56) and visualizeTree
// draws (src/HashedOctree.cpp:939-974).
// Returns the node count, -1 if cap is too small, -2 if the guard refuses the input.
long ref_build_nodes(const double* pos3, const double* mass, size_t n, const double* center3, double edge,
                     size_t cap, uint64_t* keys, int64_t* counts, double* masses, double* bary3,
                     uint8_t* childbyte, double* quad6, double* box4) {
  if (ref_guard(pos3, n, center3, edge) != 0) return -2;
  Body* b = make_bodies(pos3, nullptr, mass, n);
  OctantBounds root(Vec3D(center3[0], center3[1], center3[2]), edge);
  LinearHashedOctree tree;
  buildLinearHashedOctreeInPlace(tree, b, n, root);
  std::vector<spatialKey> order;
  order.reserve(tree.nodes.size());
  for (auto& kv : tree.nodes) order.push_back(kv.first);
  std::sort(order.begin(), order.end());
  long m = (long)order.size();
  if ((size_t)m > cap) {
    tree.deleteTree();
    delete[] b;
    return -1;
  }
  for (long j = 0; j < m; ++j) {
    HOTNode* nd = tree.lookUpNode(order[j]);
    keys[j] = nd->nodeKey;
    counts[j] = nd->N;
    masses[j] = nd->mass;
    bary3[3 * j] = nd->baryCenter.x;
    bary3[3 * j + 1] = nd->baryCenter.y;
    bary3[3 * j + 2] = nd->baryCenter.z;
    childbyte[j] = nd->childByte;
    for (int q = 0; q < 6; ++q) quad6[6 * j + q] = nd->quadrupoleMoment[q];
    if (box4) {
      box4[4 * j] = nd->nodeBounds.center.x;
      box4[4 * j + 1] = nd->nodeBounds.center.y;
      box4[4 * j + 2] = nd->nodeBounds.center.z;
      box4[4 * j + 3] = nd->nodeBounds.size;
    }
  }
  tree.deleteTree();
  delete[] b;
  return m;
}

// Tree build plus ComputeHOTOctreeForce on zeroed accelerations (as ofApp does after
// ResetVec3D). list_len (optional) receives each body's interaction-list length.
int ref_force(const double* pos3, const double* mass, size_t n, const double* center3, double edge, double theta,
              double* acc3, int64_t* list_len) {
  if (ref_guard(pos3, n, center3, edge) != 0) return -2;
  Body* b = make_bodies(pos3, nullptr, mass, n);
  OctantBounds root(Vec3D(center3[0], center3[1], center3[2]), edge);
  LinearHashedOctree tree;
  buildLinearHashedOctreeInPlace(tree, b, n, root);
  Vec3D* acc = new Vec3D[n];
  HOTNode** walk = new HOTNode*[n + 1];
  HOTNode** inter = new HOTNode*[n + 1];
  ComputeHOTOctreeForce(tree, b, acc, n, walk, inter, theta);
  for (size_t i = 0; i < n; ++i) {
    acc3[3 * i] = acc[i].x;
    acc3[3 * i + 1] = acc[i].y;
    acc3[3 * i + 2] = acc[i].z;
  }
  if (list_len)
    for (size_t i = 0; i < n; ++i) list_len[i] = TraverseHOTInteractionList(tree, b[i].position, theta, walk, inter);
  delete[] walk;
  delete[] inter;
  delete[] acc;
  tree.deleteTree();
  delete[] b;
  return 0;
}

// nsteps frames of ofApp::update()+draw() (drawing excluded). pos/vel/mass are updated in
// place and left in the reference's body order; acc3 carries the app's acceleration array,
// which RadixSortBodies does not reorder. edge_factor scales the root edge handed to the
// build (1 = the app's literal bounds). stage_s (optional, 6 doubles) accumulates seconds
// for: bounds+keys, sort, kick+drift, build, force, kick+free. perm_out (optional) gets the
// composed permutation (slot -> original index).
int ref_app_steps(double* pos3, double* vel3, double* mass, size_t n, double dt, double theta, double edge_factor,
                  int nsteps, double* acc3, double* stage_s, uint32_t* perm_out) {
  Body* b = make_bodies(pos3, vel3, mass, n);
  Vec3D* acc = new Vec3D[n];
  for (size_t i = 0; i < n; ++i) acc[i] = Vec3D(acc3[3 * i], acc3[3 * i + 1], acc3[3 * i + 2]);
  LinearHashedOctree tree;
  int rc = 0;
  for (int s = 0; s < nsteps; ++s) {
    double t0 = now_s();
    OctantBounds rb(b, n);
    for (size_t i = 0; i < n; ++i) b[i].bodyKey = computeMortonKey(b[i].position, rb.size);
    double t1 = now_s();
    RadixSortBodies(b, n);
    double t2 = now_s();
    ComputePositionAtHalfTimeStep(dt, b, n, acc);
    double t3 = now_s();
    OctantBounds tb(rb.center, rb.size * edge_factor);
    {
      std::vector<double> p(3 * n);
      for (size_t i = 0; i < n; ++i) {
        p[3 * i] = b[i].position.x;
        p[3 * i + 1] = b[i].position.y;
        p[3 * i + 2] = b[i].position.z;
      }
      double c[3] = {tb.center.x, tb.center.y, tb.center.z};
      if (ref_guard(p.data(), n, c, tb.size) != 0) {
        rc = -2;
        break;
      }
    }
    double t3g = now_s();
    buildLinearHashedOctreeInPlace(tree, b, n, tb);
    double t4 = now_s();
    HOTNode** walk = new HOTNode*[n + 1];
    HOTNode** inter = new HOTNode*[n + 1];
    ResetVec3D(acc, (int)n);
    ComputeHOTOctreeForce(tree, b, acc, n, walk, inter, theta);
    double t5 = now_s();
    ComputeVelocityAndPosition(dt, b, n, acc);
    delete[] walk;
    delete[] inter;
    tree.deleteTree();
    double t6 = now_s();
    if (stage_s) {
      stage_s[0] += t1 - t0;
      stage_s[1] += t2 - t1;
      stage_s[2] += t3 - t2;
      stage_s[3] += t4 - t3g;
      stage_s[4] += t5 - t4;
      stage_s[5] += t6 - t5;
    }
  }
  for (size_t i = 0; i < n; ++i) {
    pos3[3 * i] = b[i].position.x;
    pos3[3 * i + 1] = b[i].position.y;
    pos3[3 * i + 2] = b[i].position.z;
    vel3[3 * i] = b[i].velocity.x;
    vel3[3 * i + 1] = b[i].velocity.y;
    vel3[3 * i + 2] = b[i].velocity.z;
    mass[i] = b[i].mass;
    acc3[3 * i] = acc[i].x;
    acc3[3 * i + 1] = acc[i].y;
    acc3[3 * i + 2] = acc[i].z;
    if (perm_out) perm_out[i] = (uint32_t)b[i].displayRadius;
  }
  delete[] acc;
  delete[] b;
  return rc;
}

}  // extern "C"
