// Reverse mode of the tree-force + kick-drift-kick step (bh_adjoint_forward / bh_step_backward).
//
// Forward map per step (h = dt / 2, a = tree acceleration):
//   v' = v_n + h a(x_n);   x_{n+1} = x_n + dt v';   v_{n+1} = v' + h a(x_{n+1}).
// Reverse of step n, given the adjoints (xb, vb) of (x_{n+1}, v_{n+1}) and the carry from step
// n+1 (h times the adjoint of its half-step velocity, i.e. the share of a(x_{n+1}) used by its
// first half-kick):
//   ab = h vb + carry;   (xb, mb) += VJP of a at x_{n+1} applied to ab;
//   vb += dt xb;   carry = h vb.
// After step 0, ab = carry and one more VJP at x_0 finishes the gradients.
//
// The VJP keeps the tree walk's opening decisions fixed: the forward walk of every step is
// re-run from a checkpoint with recording on (each flushed 32-entry interaction buffer is
// appended, with its lane masks, to a tape), and the VJP kernel replays exactly those entries:
//   point  j -> i:  t = m_j w3 d,  d = x_j - x_i,  w_k = (d^2 + eps^2)^(-k/2)
//                   dt/dd^T ab = m_j (w3 ab - 3 w5 (ab.d) d);  xb_i -= it, xb_j += it,
//                   mb_j += w3 ab.d
//   cell   c -> i:  t = M w3 d - w5 Q d + 2.5 w7 (d.Q.d) d,  d = C - x_i
//                   xb_i -= g, and the node collects (Cb, Mb, Qb) += (g, w3 ab.d, dt/dQ . ab)
// with g = ab (M w3 + 2.5 w7 s) + d (-3 M w5 (ab.d) + 5 w7 (ab.Q.d) - 17.5 w9 s (ab.d))
//          + 5 w7 (ab.d) Q d - w5 Q ab,   s = d.Q.d.
// A node's (C, M, Q) are its members' centre of mass, mass and quadrupole about C, so the node
// adjoints reach each member body k (r = x_k - C, symmetric Gs from Qb):
//   xb_k += (m_k / M) Cb + m_k (6 Gs r - 2 tr(Gs) r)
//   mb_k += Mb + Cb.r / M + 3 r.Gs.r - r^2 tr(Gs)      (dQ/dC = 0 because sum m r = 0).
// Positions and velocities stay in upload order on this path (no Morton reordering), so every
// per-body array is indexed by body id.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 256;
constexpr int kNadj = 12;  // floats per node adjoint: Cb (3), Mb, Qb (6), pad (2)

struct TapeSlot {
  WalkNode* wn = nullptr;
  float4* tpos = nullptr;
  uint32_t* tslot = nullptr;
  Chunk* chunks = nullptr;
  unsigned* count = nullptr;  // device
  size_t node_cap = 0;
  size_t chunk_cap = 0;
  int m = 0;
  unsigned nchunks = 0;
};

struct AdjState {
  bh_params prm{};
  int nsteps = 0;
  int every = 1;
  int nck = 0;
  size_t n = 0;
  float4* ck = nullptr;  // [nck + 1][3][n]: x, v, a at steps 0, every, 2 every, ..., then the final state
  int final_slot = 0;
  std::vector<TapeSlot> tape;
  size_t chunk_cap = 0;
  float4* xbar = nullptr;
  float4* vbar = nullptr;
  float4* carry = nullptr;
  float4* abar = nullptr;
  float* mbar = nullptr;
  float* nadj = nullptr;
  size_t nadj_cap = 0;
  unsigned* next = nullptr;
  bool valid = false;
  bool vjp_attr = false;
  int vjp_blocks_per_sm = 0;  // resident k_vjp blocks per SM (queried once)
};

__global__ void k_adj_abar(const float4* __restrict__ vbar, const float4* __restrict__ carry, float h, int n,
                           float4* __restrict__ abar) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const float4 v = vbar[i], c = carry[i];
  abar[i] = make_float4(fmaf(h, v.x, c.x), fmaf(h, v.y, c.y), fmaf(h, v.z, c.z), 0.f);
}

__global__ void k_adj_vupdate(float4* __restrict__ vbar, const float4* __restrict__ xbar, float dt, float h, int n,
                              float4* __restrict__ carry) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  float4 v = vbar[i];
  const float4 x = xbar[i];
  v.x = fmaf(dt, x.x, v.x);
  v.y = fmaf(dt, x.y, v.y);
  v.z = fmaf(dt, x.z, v.z);
  vbar[i] = v;
  carry[i] = make_float4(h * v.x, h * v.y, h * v.z, 0.f);
}

// Per-warp shared memory of the replay: the group's bodies and their acceleration adjoints, and
// a 16 x 32 table (padded rows, conflict-free both ways) of body-side terms for each axis: the
// bodies are taken 16 at a time, which halves the table and doubles the resident warps.
constexpr int kVjpHalf = 16;
struct VjpWarp {
  float4 pos[32];
  float4 ab[32];
  float g[3][kVjpHalf][33];
};

// Lane b of the half [h, h + 16) sums its body's row over the chunk's entries; d = source -
// body, so the body's own position takes the negative.
__device__ __forceinline__ void vjp_rows(VjpWarp& s, int h, int hend, int lane, int cnt, uint32_t my_slot,
                                         float4* __restrict__ xbar) {
  __syncwarp();
  if (lane >= h && lane < hend) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int k = 0; k < cnt; ++k) {
      sx += s.g[0][lane - h][k];
      sy += s.g[1][lane - h][k];
      sz += s.g[2][lane - h][k];
    }
    atomicAdd(&xbar[my_slot].x, -sx);
    atomicAdd(&xbar[my_slot].y, -sy);
    atomicAdd(&xbar[my_slot].z, -sz);
  }
  __syncwarp();
}

constexpr int kVjpWarps = 4;
constexpr size_t kVjpSmem = sizeof(VjpWarp) * kVjpWarps;

// Replays the recorded chunks, one warp per chunk, lane = buffer entry: each lane loops over the
// group's bodies, sums its entry's adjoints (node or source body) in registers and leaves the
// body-side term in the table; then lane b sums row b for body b.
__global__ __launch_bounds__(kVjpWarps * 32) void k_vjp(const Chunk* __restrict__ chunks, unsigned nchunks,
                                                        const WalkNode* __restrict__ nodes,
                                                        const float4* __restrict__ tpos,
                                                        const uint32_t* __restrict__ tslot,
                                                        const float4* __restrict__ abar, float eps2,
                                                        float4* __restrict__ xbar, float* __restrict__ mbar,
                                                        float* __restrict__ nadj, unsigned* __restrict__ next) {
  extern __shared__ __align__(16) unsigned char vjp_smem[];
  VjpWarp& s = reinterpret_cast<VjpWarp*>(vjp_smem)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned q = 0;
    if (lane == 0) q = atomicAdd(next, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nchunks) break;
    const int4 hdr = chunks[q].hdr;
    const int gbase = hdr.x, gcount = hdr.y, kind = hdr.z, cnt = hdr.w;
    __syncwarp();
    uint32_t my_slot = 0;
    if (lane < gcount) {
      my_slot = tslot[gbase + lane];
      s.pos[lane] = tpos[gbase + lane];
      s.ab[lane] = abar[my_slot];
    }
    const bool has = lane < cnt;
    const int e = has ? chunks[q].idx[lane] : 0;
    const uint32_t mk = has ? chunks[q].mask[lane] : 0u;
    __syncwarp();
    if (kind == 0) {
      const WalkNode& nd = nodes[e];
      const float4 C = nd.mac, B = nd.mq, Q2 = nd.q2;
      const float M = B.x, qxx = B.y, qxy = B.z, qxz = B.w, qyy = Q2.x, qyz = Q2.y, qzz = Q2.z;
      float cbx = 0.f, cby = 0.f, cbz = 0.f, mb = 0.f;
      float bxx = 0.f, bxy = 0.f, bxz = 0.f, byy = 0.f, byz = 0.f, bzz = 0.f;
      for (int h = 0; h < gcount; h += kVjpHalf) {
      const int hend = min(h + kVjpHalf, gcount);
      for (int b = h; b < hend; ++b) {
        const float4 p = s.pos[b], ab = s.ab[b];
        const bool take = (mk >> b) & 1u;
        const float dx = C.x - p.x, dy = C.y - p.y, dz = C.z - p.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
        const float rinv = rsqrtf(r2);
        const float u = rinv * rinv;
        const float w3 = rinv * u, w5 = w3 * u, w7 = w5 * u, w9 = w7 * u;
        const float Qdx = fmaf(qxx, dx, fmaf(qxy, dy, qxz * dz));
        const float Qdy = fmaf(qxy, dx, fmaf(qyy, dy, qyz * dz));
        const float Qdz = fmaf(qxz, dx, fmaf(qyz, dy, qzz * dz));
        const float Qax = fmaf(qxx, ab.x, fmaf(qxy, ab.y, qxz * ab.z));
        const float Qay = fmaf(qxy, ab.x, fmaf(qyy, ab.y, qyz * ab.z));
        const float Qaz = fmaf(qxz, ab.x, fmaf(qyz, ab.y, qzz * ab.z));
        const float sq = fmaf(dx, Qdx, fmaf(dy, Qdy, dz * Qdz));
        const float ad = take ? fmaf(ab.x, dx, fmaf(ab.y, dy, ab.z * dz)) : 0.f;
        const float aQd = fmaf(ab.x, Qdx, fmaf(ab.y, Qdy, ab.z * Qdz));
        const float ca = take ? fmaf(M, w3, 2.5f * w7 * sq) : 0.f;
        const float cd = fmaf(-3.f * M, w5 * ad, fmaf(take ? 5.f * w7 : 0.f, aQd, -17.5f * w9 * sq * ad));
        const float cq = 5.f * w7 * ad;
        const float w5t = take ? w5 : 0.f;
        const float gx = fmaf(ca, ab.x, fmaf(cd, dx, fmaf(cq, Qdx, -w5t * Qax)));
        const float gy = fmaf(ca, ab.y, fmaf(cd, dy, fmaf(cq, Qdy, -w5t * Qay)));
        const float gz = fmaf(ca, ab.z, fmaf(cd, dz, fmaf(cq, Qdz, -w5t * Qaz)));
        s.g[0][b - h][lane] = gx;
        s.g[1][b - h][lane] = gy;
        s.g[2][b - h][lane] = gz;
        cbx += gx;
        cby += gy;
        cbz += gz;
        mb = fmaf(w3, ad, mb);
        const float h25 = 2.5f * w7 * ad;
        const float ax = take ? ab.x : 0.f, ay = take ? ab.y : 0.f, az = take ? ab.z : 0.f;
        bxx += fmaf(-w5 * ax, dx, h25 * dx * dx);
        byy += fmaf(-w5 * ay, dy, h25 * dy * dy);
        bzz += fmaf(-w5 * az, dz, h25 * dz * dz);
        bxy += fmaf(-w5, fmaf(ax, dy, ay * dx), 2.f * h25 * dx * dy);
        bxz += fmaf(-w5, fmaf(ax, dz, az * dx), 2.f * h25 * dx * dz);
        byz += fmaf(-w5, fmaf(ay, dz, az * dy), 2.f * h25 * dy * dz);
      }
      vjp_rows(s, h, hend, lane, cnt, my_slot, xbar);
      }
      if (has && mk) {
        float* a = nadj + (size_t)e * kNadj;
        atomicAdd(a + 0, cbx);
        atomicAdd(a + 1, cby);
        atomicAdd(a + 2, cbz);
        atomicAdd(a + 3, mb);
        atomicAdd(a + 4, bxx);
        atomicAdd(a + 5, bxy);
        atomicAdd(a + 6, bxz);
        atomicAdd(a + 7, byy);
        atomicAdd(a + 8, byz);
        atomicAdd(a + 9, bzz);
      }
    } else {
      const int src = has ? (e >= 0 ? e : nodes[-e - 1].link.z) : 0;  // a point node is a single-body leaf
      const float4 v = tpos[src];
      float tx = 0.f, ty = 0.f, tz = 0.f, tm = 0.f;
      for (int h = 0; h < gcount; h += kVjpHalf) {
      const int hend = min(h + kVjpHalf, gcount);
      for (int b = h; b < hend; ++b) {
        const float4 p = s.pos[b], ab = s.ab[b];
        const bool take = ((mk >> b) & 1u) && src != gbase + b;
        const float dx = v.x - p.x, dy = v.y - p.y, dz = v.z - p.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
        const float rinv = rsqrtf(r2);
        const float w3 = take ? rinv * rinv * rinv : 0.f;
        const float w5 = w3 * rinv * rinv;
        const float ad = fmaf(ab.x, dx, fmaf(ab.y, dy, ab.z * dz));
        const float k3 = -3.f * w5 * ad;
        const float gx = v.w * fmaf(w3, ab.x, k3 * dx);
        const float gy = v.w * fmaf(w3, ab.y, k3 * dy);
        const float gz = v.w * fmaf(w3, ab.z, k3 * dz);
        s.g[0][b - h][lane] = gx;
        s.g[1][b - h][lane] = gy;
        s.g[2][b - h][lane] = gz;
        tx += gx;
        ty += gy;
        tz += gz;
        tm = fmaf(w3, ad, tm);
      }
      vjp_rows(s, h, hend, lane, cnt, my_slot, xbar);
      }
      if (has && mk) {
        const uint32_t ss = tslot[src];
        atomicAdd(&xbar[ss].x, tx);
        atomicAdd(&xbar[ss].y, ty);
        atomicAdd(&xbar[ss].z, tz);
        atomicAdd(&mbar[ss], tm);
      }
    }
  }
}

// Node adjoints -> member bodies: each body walks from the root to its leaf and adds the share
// of every multi-body node on the way.
__global__ __launch_bounds__(kThreads) void k_nadj_bodies(const WalkNode* __restrict__ nodes,
                                                          const float4* __restrict__ tpos,
                                                          const uint32_t* __restrict__ tslot,
                                                          const float* __restrict__ nadj, int n,
                                                          float4* __restrict__ xbar, float* __restrict__ mbar) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const float4 x = tpos[i];
  float xb0 = 0.f, xb1 = 0.f, xb2 = 0.f, mb = 0.f;
  int node = 0;
  for (int depth = 0; depth <= kMaxDepth; ++depth) {
    const int4 link = nodes[node].link;
    if (link.w > 1) {
      const float* a = nadj + (size_t)node * kNadj;
      const float cbx = a[0], cby = a[1], cbz = a[2], Mb = a[3];
      const float gxx = a[4], gxy = 0.5f * a[5], gxz = 0.5f * a[6], gyy = a[7], gyz = 0.5f * a[8], gzz = a[9];
      const float4 C = nodes[node].mac;
      const float M = nodes[node].mq.x;
      const float rx = x.x - C.x, ry = x.y - C.y, rz = x.z - C.z;
      const float grx = fmaf(gxx, rx, fmaf(gxy, ry, gxz * rz));
      const float gry = fmaf(gxy, rx, fmaf(gyy, ry, gyz * rz));
      const float grz = fmaf(gxz, rx, fmaf(gyz, ry, gzz * rz));
      const float tr = gxx + gyy + gzz;
      const float mM = x.w / M;
      xb0 += fmaf(mM, cbx, x.w * fmaf(6.f, grx, -2.f * tr * rx));
      xb1 += fmaf(mM, cby, x.w * fmaf(6.f, gry, -2.f * tr * ry));
      xb2 += fmaf(mM, cbz, x.w * fmaf(6.f, grz, -2.f * tr * rz));
      const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
      mb += Mb + fmaf(cbx, rx, fmaf(cby, ry, cbz * rz)) / M + fmaf(3.f, fmaf(rx, grx, fmaf(ry, gry, rz * grz)), -r2 * tr);
    }
    if (link.y == 0) break;
    int next = -1;
    for (int c = link.x; c < link.x + link.y; ++c) {
      const int4 cl = nodes[c].link;
      if (i >= cl.z && i < cl.z + cl.w) {
        next = c;
        break;
      }
    }
    if (next < 0) break;
    node = next;
  }
  const uint32_t slot = tslot[i];
  float4 xb = xbar[slot];
  xb.x += xb0;
  xb.y += xb1;
  xb.z += xb2;
  xbar[slot] = xb;
  mbar[slot] += mb;
}

inline int grid_for(long long n) { return (int)((n + kThreads - 1) / kThreads); }

AdjState* state(bh_ctx* c) { return reinterpret_cast<AdjState*>(c->adj); }

void free_slot(TapeSlot& t) {
  dfree(t.wn);
  dfree(t.tpos);
  dfree(t.tslot);
  dfree(t.chunks);
  dfree(t.count);
  t = TapeSlot();
}

bh_status ensure_slot(TapeSlot& t, size_t n, size_t node_cap, size_t chunk_cap) {
  if (t.node_cap < node_cap) {
    dfree(t.wn);
    t.node_cap = 0;
    BH_TRY(dalloc(&t.wn, node_cap));
    t.node_cap = node_cap;
  }
  if (!t.tpos) BH_TRY(dalloc(&t.tpos, n));
  if (!t.tslot) BH_TRY(dalloc(&t.tslot, n));
  if (!t.count) BH_TRY(dalloc(&t.count, 1));
  if (t.chunk_cap < chunk_cap) {
    dfree(t.chunks);
    t.chunk_cap = 0;
    BH_TRY(dalloc(&t.chunks, chunk_cap));
    t.chunk_cap = chunk_cap;
  }
  return BH_OK;
}

// Bounds of the current positions -> tree -> multipoles (the geometry of bh_build with
// edge = edge_factor * size), then the acceleration walk into c->acc; recorded into `rec`
// when given. Used for a(x_0) of the differentiable path.
bh_status force_at_current(bh_ctx* c, const bh_params& p, TapeSlot* rec) {
  const int n = (int)c->n;
  for (;;) {
    clear_device_flags(c);
    launch_bounds(c, c->pos[c->cur], n, p.edge_factor);
    launch_treekey(c, c->pos[c->cur], n, c->tkey, c->tslot);
    uint64_t* ko;
    uint32_t* vo;
    radix_sort_pairs(c, c->tkey, c->tslot, c->keys[1], c->vals[1], n, c->stream, &ko, &vo);
    launch_gather_tree(c, c->tslot, n, c->pos[c->cur], c->tpos);
    launch_build(c, n, p.leaf_capacity);
    launch_upsweep(c, n, p.leaf_capacity, BH_MULTIPOLE_QUADRUPOLE);
    if (rec) {
      cudaMemsetAsync(rec->count, 0, sizeof(unsigned), c->stream);
      launch_walk_record(c, n, (float)p.theta, (float)p.eps, c->acc, nullptr, 0.f, rec->chunks, rec->count,
                         (int)rec->chunk_cap);
    } else {
      launch_walk(c, n, (float)p.theta, (float)p.eps, BH_MULTIPOLE_QUADRUPOLE, c->acc, nullptr, 0.f);
    }
    BH_TRY(last_launch());
    uint32_t e = 0;
    BH_TRY(sync_and_check(c, &e));
    if (e & kErrNodes) {
      BH_TRY(ensure_nodes(c, c->node_cap * 2));
      continue;
    }
    if (e) return err_to_status(e);
    return BH_OK;
  }
}

// One step of the differentiable path (bodies keep their order). With rec, the walk records
// its interaction buffers and the tree (walk records, tree-order positions, permutation) is
// copied into the tape slot.
bh_status fixed_step(bh_ctx* c, const bh_params& p, TapeSlot* rec) {
  const int n = (int)c->n;
  const float dt = (float)p.dt;
  for (;;) {
    const int nx = 1 - c->cur;
    clear_device_flags(c);
    launch_bounds(c, c->pos[c->cur], n, p.edge_factor);
    launch_gather_kd_treekey(c, nullptr, n, c->pos[c->cur], c->vel[c->cur], c->acc, 1, dt, c->pos[nx], c->vel[nx],
                             c->tkey, c->tslot);
    uint64_t* ko;
    uint32_t* vo;
    radix_sort_pairs(c, c->tkey, c->tslot, c->keys[1], c->vals[1], n, c->stream, &ko, &vo);
    launch_gather_tree(c, c->tslot, n, c->pos[nx], c->tpos);
    launch_build(c, n, p.leaf_capacity);
    launch_upsweep(c, n, p.leaf_capacity, BH_MULTIPOLE_QUADRUPOLE);
    if (rec) {
      cudaMemsetAsync(rec->count, 0, sizeof(unsigned), c->stream);
      launch_walk_record(c, n, (float)p.theta, (float)p.eps, c->acc, c->vel[nx], 0.5f * dt, rec->chunks, rec->count,
                         (int)rec->chunk_cap);
    } else {
      launch_walk(c, n, (float)p.theta, (float)p.eps, BH_MULTIPOLE_QUADRUPOLE, c->acc, c->vel[nx], 0.5f * dt);
    }
    BH_TRY(last_launch());
    uint32_t e = 0;
    BH_TRY(sync_and_check(c, &e));
    if (e & kErrNodes) {
      BH_TRY(ensure_nodes(c, c->node_cap * 2));
      continue;
    }
    if (e) return err_to_status(e);
    c->cur = nx;
    return BH_OK;
  }
}

// Copies the tree of the last force evaluation into the tape slot (the chunks are already there).
bh_status capture_tree(bh_ctx* c, TapeSlot& t) {
  const int m = c->h_level_bounds[kLevels];
  const int n = (int)c->n;
  if ((size_t)m > t.node_cap) {
    dfree(t.wn);
    t.node_cap = 0;
    BH_TRY(dalloc(&t.wn, (size_t)m));
    t.node_cap = (size_t)m;
  }
  cudaMemcpyAsync(t.wn, c->wnode, sizeof(WalkNode) * m, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(t.tpos, c->tpos, sizeof(float4) * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(t.tslot, c->tslot, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(&t.nchunks, t.count, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
  BH_TRY(cuda_status(cudaStreamSynchronize(c->stream)));
  t.m = m;
  return BH_OK;
}

// Records the step (or the initial force when step == false) into slot t, growing the chunk
// capacity and redoing it when the tape overflows. The state is restored by the caller-provided
// snapshot before a redo (the step is transactional through the ping-pong buffers).
bh_status record_into(bh_ctx* c, AdjState* a, TapeSlot& t, bool step) {
  for (;;) {
    BH_TRY(ensure_slot(t, c->n, c->node_cap, a->chunk_cap));
    const bh_status s = step ? fixed_step(c, a->prm, &t) : force_at_current(c, a->prm, &t);
    if (s == BH_ERR_OVERFLOW_TAPE) {
      a->chunk_cap *= 2;
      continue;
    }
    BH_TRY(s);
    return capture_tree(c, t);
  }
}

// (xbar, mbar) += VJP of the tree acceleration recorded in t, applied to a->abar.
bh_status vjp(bh_ctx* c, AdjState* a, const TapeSlot& t) {
  const int n = (int)c->n;
  if ((size_t)t.m > a->nadj_cap) {
    dfree(a->nadj);
    a->nadj_cap = 0;
    BH_TRY(dalloc(&a->nadj, (size_t)t.m * kNadj));
    a->nadj_cap = (size_t)t.m;
  }
  cudaMemsetAsync(a->nadj, 0, sizeof(float) * kNadj * (size_t)t.m, c->stream);
  cudaMemsetAsync(a->next, 0, sizeof(unsigned), c->stream);
  const int sms = c->sms;
  if (!a->vjp_attr) {
    BH_TRY(cuda_status(cudaFuncSetAttribute(k_vjp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kVjpSmem)));
    int per_sm = 0;
    BH_TRY(cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vjp, kVjpWarps * 32, kVjpSmem)));
    a->vjp_blocks_per_sm = std::max(1, per_sm);
    a->vjp_attr = true;
  }
  // every resident block of four warps (30 KB of shared memory each)
  const int grid = std::max(1, std::min(sms * a->vjp_blocks_per_sm, (int)(t.nchunks / kVjpWarps) + 1));
  const float eps2 = (float)(a->prm.eps * a->prm.eps);
  c->launches += 2;
  if (t.nchunks > 0)
    k_vjp<<<grid, kVjpWarps * 32, kVjpSmem, c->stream>>>(t.chunks, t.nchunks, t.wn, t.tpos, t.tslot, a->abar, eps2,
                                                          a->xbar, a->mbar, a->nadj, a->next);
  k_nadj_bodies<<<grid_for(n), kThreads, 0, c->stream>>>(t.wn, t.tpos, t.tslot, a->nadj, n, a->xbar, a->mbar);
  return last_launch();
}

float4* ck_ptr(AdjState* a, int k, int which) { return a->ck + ((size_t)k * 3 + which) * a->n; }

bh_status restore_checkpoint(bh_ctx* c, AdjState* a, int k) {
  const size_t bytes = sizeof(float4) * a->n;
  c->cur = 0;
  cudaMemcpyAsync(c->pos[0], ck_ptr(a, k, 0), bytes, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->vel[0], ck_ptr(a, k, 1), bytes, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->acc, ck_ptr(a, k, 2), bytes, cudaMemcpyDeviceToDevice, c->stream);
  return last_launch();
}

}  // namespace

void adj_invalidate(bh_ctx* c) {
  if (c->adj) state(c)->valid = false;
}

void adj_release(bh_ctx* c) {
  AdjState* a = state(c);
  if (!a) return;
  for (auto& t : a->tape) free_slot(t);
  dfree(a->ck);
  dfree(a->xbar);
  dfree(a->vbar);
  dfree(a->carry);
  dfree(a->abar);
  dfree(a->mbar);
  dfree(a->nadj);
  dfree(a->next);
  delete a;
  c->adj = nullptr;
}

}  // namespace bh

using namespace bh;

extern "C" {

bh_status bh_adjoint_forward(bh_ctx* c, const bh_params* p, int nsteps, int checkpoint_every, bh_stats* st) {
  bh::Range range_("bh_adjoint_forward");
  if (!c || !p || nsteps < 1 || checkpoint_every < 1 || c->batch || c->n == 0 ||
      p->multipole != BH_MULTIPOLE_QUADRUPOLE || !(p->eps > 0) || !(p->theta >= 0) || p->leaf_capacity < 1 ||
      !(p->edge_factor > 0))
    return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (st) std::memset(st, 0, sizeof(*st));
  if (!c->adj) c->adj = new AdjState();
  AdjState* a = state(c);
  a->valid = false;
  a->prm = *p;
  a->prm.acc_follows_body = 1;
  a->nsteps = nsteps;
  a->every = checkpoint_every;
  const int nck = (nsteps + checkpoint_every - 1) / checkpoint_every;
  if (a->n != c->n || a->nck < nck) {
    dfree(a->ck);
    for (auto& t : a->tape) free_slot(t);
    a->tape.clear();
    dfree(a->xbar);
    dfree(a->vbar);
    dfree(a->carry);
    dfree(a->abar);
    dfree(a->mbar);
    a->nck = 0;
    a->n = c->n;
    BH_TRY(dalloc(&a->ck, (size_t)(nck + 1) * 3 * c->n));
    BH_TRY(dalloc(&a->xbar, c->n));
    BH_TRY(dalloc(&a->vbar, c->n));
    BH_TRY(dalloc(&a->carry, c->n));
    BH_TRY(dalloc(&a->abar, c->n));
    BH_TRY(dalloc(&a->mbar, c->n));
    if (!a->next) BH_TRY(dalloc(&a->next, 1));
    a->nck = nck;
  }
  BH_TRY(ensure_nodes(c, std::max<size_t>(2 * c->n + 64, 1024)));
  // a(x_0), recorded once to size the tape
  if (a->chunk_cap == 0) a->chunk_cap = (c->n / 32 + 1) * 64;
  if (a->tape.size() < 1) a->tape.resize(1);
  cudaEvent_t e0 = c->stage_ev[0], e1 = c->stage_ev[1];
  const uint64_t launches0 = c->launches;
  cudaEventRecord(e0, c->stream);
  BH_TRY(record_into(c, a, a->tape[0], false));
  a->chunk_cap = std::max<size_t>(a->chunk_cap, (size_t)(a->tape[0].nchunks * 1.5) + 1024);
  const size_t bytes = sizeof(float4) * c->n;
  for (int s = 0; s < nsteps; ++s) {
    if (s % checkpoint_every == 0) {
      const int k = s / checkpoint_every;
      cudaMemcpyAsync(ck_ptr(a, k, 0), c->pos[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream);
      cudaMemcpyAsync(ck_ptr(a, k, 1), c->vel[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream);
      cudaMemcpyAsync(ck_ptr(a, k, 2), c->acc, bytes, cudaMemcpyDeviceToDevice, c->stream);
    }
    BH_TRY(fixed_step(c, a->prm, nullptr));
    if (st) {
      st->interactions_cell += c->h_counters->cell;
      st->interactions_p2p += c->h_counters->p2p;
    }
  }
  a->final_slot = nck;
  cudaMemcpyAsync(ck_ptr(a, nck, 0), c->pos[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(ck_ptr(a, nck, 1), c->vel[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(ck_ptr(a, nck, 2), c->acc, bytes, cudaMemcpyDeviceToDevice, c->stream);
  cudaEventRecord(e1, c->stream);
  BH_TRY(cuda_status(cudaEventSynchronize(e1)));
  if (st) {
    st->ms_step = elapsed(c, 0, 1);
    st->steps = (uint32_t)nsteps;
    st->kernel_launches = (uint32_t)(c->launches - launches0);
  }
  a->valid = true;
  c->tree_valid = false;
  return BH_OK;
}

bh_status bh_step_backward(bh_ctx* c, const float* dl_dx4, const float* dl_dv4, float* grad_x4, float* grad_v4,
                           float* grad_m, bh_stats* st) {
  bh::Range range_("bh_step_backward");
  if (!c || !c->adj) return BH_ERR_INVALID_ARG;
  AdjState* a = state(c);
  if (!a->valid || a->n != c->n) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (st) std::memset(st, 0, sizeof(*st));
  const int n = (int)c->n;
  const size_t bytes = sizeof(float4) * n;
  const uint64_t launches0 = c->launches;
  cudaEventRecord(c->stage_ev[0], c->stream);
  if (dl_dx4)
    cudaMemcpyAsync(a->xbar, dl_dx4, bytes, cudaMemcpyHostToDevice, c->stream);
  else
    cudaMemsetAsync(a->xbar, 0, bytes, c->stream);
  if (dl_dv4)
    cudaMemcpyAsync(a->vbar, dl_dv4, bytes, cudaMemcpyHostToDevice, c->stream);
  else
    cudaMemsetAsync(a->vbar, 0, bytes, c->stream);
  cudaMemsetAsync(a->carry, 0, bytes, c->stream);
  cudaMemsetAsync(a->mbar, 0, sizeof(float) * n, c->stream);
  const float dt = (float)a->prm.dt, h = 0.5f * dt;
  const int every = a->every;
  if ((int)a->tape.size() < every) a->tape.resize(every);
  const int nseg = (a->nsteps + every - 1) / every;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * every, s1 = std::min(s0 + every, a->nsteps);
    BH_TRY(restore_checkpoint(c, a, seg));
    for (int t = 0; t < s1 - s0; ++t) BH_TRY(record_into(c, a, a->tape[t], true));
    for (int stp = s1 - 1; stp >= s0; --stp) {
      const TapeSlot& t = a->tape[stp - s0];
      k_adj_abar<<<grid_for(n), kThreads, 0, c->stream>>>(a->vbar, a->carry, h, n, a->abar);
      BH_TRY(vjp(c, a, t));
      k_adj_vupdate<<<grid_for(n), kThreads, 0, c->stream>>>(a->vbar, a->xbar, dt, h, n, a->carry);
      c->launches += 2;
    }
  }
  // a(x_0): the carry is its adjoint
  BH_TRY(restore_checkpoint(c, a, 0));
  BH_TRY(record_into(c, a, a->tape[0], false));
  cudaMemcpyAsync(a->abar, a->carry, bytes, cudaMemcpyDeviceToDevice, c->stream);
  BH_TRY(vjp(c, a, a->tape[0]));
  if (grad_x4) cudaMemcpyAsync(grad_x4, a->xbar, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (grad_v4) cudaMemcpyAsync(grad_v4, a->vbar, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (grad_m) cudaMemcpyAsync(grad_m, a->mbar, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
  // the bodies go back to the state after the forward pass
  BH_TRY(restore_checkpoint(c, a, a->final_slot));
  cudaEventRecord(c->stage_ev[1], c->stream);
  BH_TRY(cuda_status(cudaStreamSynchronize(c->stream)));
  if (st) {
    st->ms_step = elapsed(c, 0, 1);
    st->steps = (uint32_t)a->nsteps;
    st->kernel_launches = (uint32_t)(c->launches - launches0);
  }
  return last_launch();
}

}  // extern "C"
