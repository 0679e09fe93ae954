// Tree walk + force: ComputeHOTOctreeForce / TraverseHOTInteractionList /
// ComputeHOTForceInteractionList / LinearHashedOctree::MAC (src/HashedOctree.hpp:262-459,
// src/HashedOctree.cpp:872-885), one warp per group of up to 32 consecutive bodies in tree order
// (32 by default; the autotuner may pick 16 or 8 for small single systems).
//
// Per-lane exactness. The reference walks each body separately: pop a node; test each
// existing child with the MAC size^2 / d^2 < theta^2 against the body; accepted children go
// to the body's interaction list, the others are pushed; a popped leaf is added unless it is
// the body itself (same position). Here the warp walks once for its 32 bodies and every stack
// entry carries the 32-bit mask of lanes for which the node is still open, so each lane ends
// up with exactly the interaction set the reference builds for its body.
//
// Traversal, per round: the warp pops stack entries until their children fill the 32 lanes,
// each lane loads one child and classifies it against the bounding box of the group's bodies:
//   accept-all  the MAC holds even at the box's nearest point -> accepted by every open lane
//   open-all    the MAC fails even at the box's farthest corner -> opened by every open lane
//   mixed       otherwise: the child is broadcast and every lane runs its own MAC (a ballot)
// (both bounds carry a 1e-5 relative margin, so they agree with the per-lane FP32 test). The
// outcomes are appended to shared-memory buffers with warp-wide prefix counts:
//   cells  : accepted nodes with more than one body — monopole + quadrupole (intended mode)
//   points : single bodies — accepted single-body leaves, the members of opened leaves, and
//            (literal mode) every accepted node as a point mass at its pseudo-barycentre
// and opened internal children are pushed with their child range, so a pop needs no load.
//
// Evaluation: a full buffer (32 entries) is staged through shared memory, one entry per lane,
// and every lane runs over all 32 entries, adding an entry's term when its bit is set in the
// entry's mask. Sums are FP32 per flush, added into Kahan-compensated per-lane totals. With a
// positive softening a point at the lane's own position contributes exactly 0, so the
// self-skip test is only compiled in for zero softening.
#include <cuda_runtime.h>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kBuf = 64;
constexpr uint32_t kChildShift = 28;  // stack entry: first_child | nchild << 28
constexpr float kMacMargin = 1e-5f;

// Launch shape of one walk variant: warps per block, resident blocks per SM the register
// allocation must allow, and the per-warp stack depth. Above
// kStack - 224 entries the warp pops one entry per round, so a full round (at most 7 new
// entries per level of the remaining depth) always fits.
template <int kBlockWarps, int kMinBlocksPerSM, int kStackDepth, int kCellForm = 0>
struct WalkCfg {
  static constexpr int kForm = kCellForm;  // cell evaluation form (eval_cells)
  static constexpr int kWarps = kBlockWarps;
  static constexpr int kThreads = 32 * kBlockWarps;
  static constexpr int kMinBlocks = kMinBlocksPerSM;
  static constexpr int kStack = kStackDepth;
  static constexpr int kStackDeep = kStackDepth - 224;
};
using CfgDefault = WalkCfg<8, 4, 384>;
constexpr int kThreads = CfgDefault::kThreads;
constexpr int kWarps = CfgDefault::kWarps;

template <int kStack>
struct WarpSmemT {
  uint32_t stk_node[kStack];
  uint32_t stk_mask[kStack];
  int cell_node[kBuf];
  uint32_t cell_mask[kBuf];
  int pt_idx[kBuf];  // >= 0: body (tree order); < 0: -(node + 1)
  uint32_t pt_mask[kBuf];
  float4 st0[32];
  float4 st1[32];
  float4 st2[32];
  int ex_first[32];
  int ex_off[32];
  uint32_t ex_mask[32];
};

struct Acc {
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  __device__ __forceinline__ void add(float bx, float by, float bz) {
    float y = bx - cx, t = sx + y;
    cx = (t - sx) - y;
    sx = t;
    y = by - cy;
    t = sy + y;
    cy = (t - sy) - y;
    sy = t;
    y = bz - cz;
    t = sz + y;
    cz = (t - sz) - y;
    sz = t;
  }
};

// Interaction recording for the adjoint: where the flushed buffers go, and the current group.
struct Rec {
  Chunk* chunks;
  unsigned* count;
  int cap;
  int gbase, gcount;
  uint32_t* err;
};

// Appends one flushed buffer (cnt entries of idx / mask, still in shared memory) to the tape.
__device__ __forceinline__ void record_chunk(const Rec& r, int kind, int cnt, const int* idx, const uint32_t* mask,
                                             int lane) {
  unsigned slot = 0;
  if (lane == 0) slot = atomicAdd(r.count, 1u);
  slot = __shfl_sync(0xffffffffu, slot, 0);
  if (slot >= (unsigned)r.cap) {
    if (lane == 0) atomicOr(r.err, kErrTape);
    return;
  }
  Chunk& ch = r.chunks[slot];
  if (lane == 0) ch.hdr = make_int4(r.gbase, r.gcount, kind, cnt);
  if (lane < cnt) {
    ch.idx[lane] = idx[lane];
    ch.mask[lane] = mask[lane];
  }
}

// 32 multipole cells (monopole + quadrupole). The lane mask rides in st2.w.
template <bool kRec, int kForm = 0, class Smem>
__device__ __forceinline__ void eval_cells(Smem& s, int cnt, const WalkNode* __restrict__ nodes,
                                           uint32_t lanebit, float px, float py, float pz, float eps2, Acc& acc,
                                           unsigned long long& ev, const Rec& rec) {
  ev += (unsigned)cnt;
  __syncwarp();
  const int lane = __ffs(lanebit) - 1;
  if (kRec) record_chunk(rec, 0, cnt, s.cell_node, s.cell_mask, lane);
  if (lane < cnt) {
    const WalkNode* nd = nodes + s.cell_node[lane];
    s.st0[lane] = __ldg(&nd->mac);
    s.st1[lane] = __ldg(&nd->mq);
    float4 q2 = __ldg(&nd->q2);
    q2.w = __uint_as_float(s.cell_mask[lane]);
    s.st2[lane] = q2;
  }
  __syncwarp();
  float bx = 0.f, by = 0.f, bz = 0.f;
  // unroll factors measured at N = 2^22: cells 2 / 4 / 8 / 12 / 16 / 32 -> walk 17.98 / 17.45 /
  // 17.71 / 17.44 / 17.37 / 17.44 ms; points 2 / 4 / 8 / 16 (cells at 16) -> 17.46 / 17.37 /
  // 17.31 / 17.67 ms
#pragma unroll 16
  for (int j = 0; j < cnt; ++j) {
    const float4 c0 = s.st0[j], c1 = s.st1[j], c2 = s.st2[j];
    const float dx = c0.x - px, dy = c0.y - py, dz = c0.z - pz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    const float rinv = rsqrtf(r2);
    const float u = rinv * rinv;   // 1 / D^2
    const float w3 = rinv * u;     // 1 / D^3
    const float w5 = w3 * u;       // 1 / D^5
    // Q.d with Q = (Qxx, Qxy, Qxz, Qyy, Qyz, Qzz) = (c1.y, c1.z, c1.w, c2.x, c2.y, c2.z)
    const float qx = fmaf(c1.y, dx, fmaf(c1.z, dy, c1.w * dz));
    const float qy = fmaf(c1.z, dx, fmaf(c2.x, dy, c2.y * dz));
    const float qz = fmaf(c1.w, dx, fmaf(c2.y, dy, c2.z * dz));
    const float qr = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
    // a += d (m / D^3 + 2.5 (d.Q.d) / D^7) - Q.d / D^5
    const float radial = fmaf(qr, w5 * (2.5f * u), c1.x * w3);
    // selects rather than a branch: every lane runs the same straight-line code
    const bool take = (__float_as_uint(c2.w) & lanebit) != 0u;
    if (kForm == 0) {
      const float tx = fmaf(-w5, qx, fmaf(radial, dx, bx));
      const float ty = fmaf(-w5, qy, fmaf(radial, dy, by));
      const float tz = fmaf(-w5, qz, fmaf(radial, dz, bz));
      bx = take ? tx : bx;
      by = take ? ty : by;
      bz = take ? tz : bz;
    } else {
      // a = w5 ((m D^2 + 2.5 (d.Q.d) / D^2) d - Q.d): one select zeroes the common factor
      const float k = fmaf(2.5f * u, qr, c1.x * r2);
      const float w5m = take ? w5 : 0.f;
      bx = fmaf(w5m, fmaf(k, dx, -qx), bx);
      by = fmaf(w5m, fmaf(k, dy, -qy), by);
      bz = fmaf(w5m, fmaf(k, dz, -qz), bz);
    }
  }
  acc.add(bx, by, bz);
}

// Up to 32 point masses. The lane mask is read from pt_mask.
template <bool kSelfTest, bool kRec, class Smem>
__device__ __forceinline__ void eval_points(Smem& s, int cnt, const WalkNode* __restrict__ nodes,
                                            const float4* __restrict__ tpos, uint32_t lanebit, float px, float py,
                                            float pz, float eps2, Acc& acc, unsigned long long& ev, const Rec& rec) {
  ev += (unsigned)cnt;
  __syncwarp();
  const int lane = __ffs(lanebit) - 1;
  if (kRec) record_chunk(rec, 1, cnt, s.pt_idx, s.pt_mask, lane);
  if (lane < cnt) {
    const int e = s.pt_idx[lane];
    float4 v;
    if (e >= 0) {
      v = __ldg(tpos + e);
    } else {
      const WalkNode* nd = nodes + (-e - 1);
      const float4 mac = __ldg(&nd->mac);
      v = make_float4(mac.x, mac.y, mac.z, __ldg(&nd->mq.x));
    }
    s.st0[lane] = v;
  }
  __syncwarp();
  float bx = 0.f, by = 0.f, bz = 0.f;
#pragma unroll 8
  for (int j = 0; j < cnt; ++j) {
    const float4 v = s.st0[j];
    const uint32_t mk = s.pt_mask[j];
    const float dx = v.x - px, dy = v.y - py, dz = v.z - pz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    const float rinv = rsqrtf(r2);
    const float mr3 = v.w * rinv * rinv * rinv;
    bool take = (mk & lanebit) != 0u;
    if (kSelfTest) take = take && !((dx == 0.f) & (dy == 0.f) & (dz == 0.f));
    // a select, not a branch (walk 17.38 -> 17.18 ms at N = 2^22): a lane outside the mask adds
    // exactly 0
    const float w = take ? mr3 : 0.f;
    bx = fmaf(w, dx, bx);
    by = fmaf(w, dy, by);
    bz = fmaf(w, dz, bz);
  }
  acc.add(bx, by, bz);
}

// Moves buffer entries [32, n) to [0, n - 32) after the first 32 were evaluated.
__device__ __forceinline__ void shift_down(int* idx, uint32_t* msk, int n, int lane) {
  __syncwarp();
  const int rest = n - 32;
  int e = 0;
  uint32_t m = 0;
  if (lane < rest) {
    e = idx[32 + lane];
    m = msk[32 + lane];
  }
  __syncwarp();
  if (lane < rest) {
    idx[lane] = e;
    msk[lane] = m;
  }
}

template <bool kQuad, bool kSelfTest, bool kRec = false, class Cfg = CfgDefault>
__global__ __launch_bounds__(Cfg::kThreads, Cfg::kMinBlocks) void k_walk(const WalkNode* __restrict__ nodes,
                                                   const float4* __restrict__ tpos,
                                                   const uint32_t* __restrict__ tslot, int n, float theta2,
                                                   float eps2, float4* __restrict__ acc_slot,
                                                   float4* __restrict__ vel_kick, float half_dt,
                                                   float4* __restrict__ vel_copy,
                                                   const int4* __restrict__ groups, int ngroups_table, int gsize,
                                                   Counters* __restrict__ ctr, uint32_t* __restrict__ err,
                                                   Chunk* __restrict__ tape = nullptr,
                                                   unsigned* __restrict__ tape_count = nullptr, int tape_cap = 0) {
  constexpr int kStack = Cfg::kStack, kStackDeep = Cfg::kStackDeep;
  __shared__ WarpSmemT<kStack> smem[Cfg::kWarps];
  const int lane = threadIdx.x & 31;
  const uint32_t lanebit = 1u << lane;
  const uint32_t lt_mask = lanebit - 1u;
  WarpSmemT<kStack>& s = smem[threadIdx.x >> 5];
  if (*((volatile uint32_t*)err) & (kErrNodes | kErrTimeout)) return;
  // work items: groups of up to 32 consecutive bodies (tree order) under one root. Without a
  // group table, group g is bodies [gsize g, gsize g + gsize) of the single tree rooted at node 0
  // (gsize <= 32; lanes beyond the group's bodies stay out of every mask); batched ensembles pass
  // (first body, body count, root node) per group.
  const int ngroups = groups ? ngroups_table : (n + gsize - 1) / gsize;
  const float acc_scale = theta2 * (1.f - kMacMargin);
  const float open_scale = theta2 * (1.f + kMacMargin);
  unsigned long long tot_cell = 0, tot_pt = 0, ev_cell = 0, ev_pt = 0;  // ev_*: warp-uniform
  bool overflow = false;

  for (;;) {
    int g = 0;
    if (lane == 0) g = (int)atomicAdd(&ctr->group_next, 1u);
    g = __shfl_sync(0xffffffffu, g, 0);
    if (g >= ngroups) break;
    int gbase, gcount, root;
    if (groups) {
      const int4 gr = __ldg(groups + g);
      gbase = gr.x;
      gcount = gr.y;
      root = gr.z;
    } else {
      gbase = g * gsize;
      gcount = min(gsize, n - gbase);
      root = 0;
    }
    const int4 root_link = __ldg(&nodes[root].link);
    const Rec rec{tape, tape_count, tape_cap, gbase, gcount, err};
    const int i = gbase + lane;
    const bool valid = lane < gcount;
    const float4 p = __ldg(tpos + (valid ? i : gbase));
    const uint32_t active = __ballot_sync(0xffffffffu, valid);
    // bounding box of the group's bodies
    float bminx = p.x, bminy = p.y, bminz = p.z, bmaxx = p.x, bmaxy = p.y, bmaxz = p.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      bminx = fminf(bminx, __shfl_xor_sync(0xffffffffu, bminx, o));
      bminy = fminf(bminy, __shfl_xor_sync(0xffffffffu, bminy, o));
      bminz = fminf(bminz, __shfl_xor_sync(0xffffffffu, bminz, o));
      bmaxx = fmaxf(bmaxx, __shfl_xor_sync(0xffffffffu, bmaxx, o));
      bmaxy = fmaxf(bmaxy, __shfl_xor_sync(0xffffffffu, bmaxy, o));
      bmaxz = fmaxf(bmaxz, __shfl_xor_sync(0xffffffffu, bmaxz, o));
    }
    Acc acc;
    int sp = 0, ncell = 0, npt = 0;
    // per-lane shares of the group's interaction counts (each lane counts the entries it
    // appended, times the lanes in their masks); self pairs are subtracted
    long long cnt_cell = 0, cnt_pt = 0;

    if (root_link.y == 0) {
      // the root is a leaf: every lane sums all its bodies
      for (int base = 0; base < root_link.w; base += 32) {
        const int k = min(32, root_link.w - base);
        __syncwarp();
        if (lane < k) {
          s.pt_idx[lane] = root_link.z + base + lane;
          s.pt_mask[lane] = active;
        }
        if (lane == 0) cnt_pt += (long long)k * __popc(active);
        eval_points<kSelfTest, kRec>(s,k, nodes, tpos, lanebit, p.x, p.y, p.z, eps2, acc, ev_pt, rec);
      }
      if (lane == 0) cnt_pt -= __popc(active);
    } else {
      __syncwarp();
      if (lane == 0) {
        s.stk_node[0] = (uint32_t)root_link.x | ((uint32_t)root_link.y << kChildShift);
        s.stk_mask[0] = active;
      }
      sp = 1;
    }

    while (sp > 0) {
      __syncwarp();
      // ---- pop entries whose children fill at most 32 lanes
      const int avail = min(sp, sp > kStackDeep ? 1 : 32);
      uint32_t ent = 0, emask = 0;
      int nch = 0;
      if (lane < avail) {
        ent = s.stk_node[sp - 1 - lane];
        emask = s.stk_mask[sp - 1 - lane];
        nch = (int)(ent >> kChildShift);
      }
      int incl = nch;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const uint32_t take = __ballot_sync(0xffffffffu, lane < avail && incl <= 32);
      const int k = __popc(take);  // >= 1: one entry has at most 8 children
      const int total = __shfl_sync(0xffffffffu, incl, k - 1);
      sp -= k;
      const int start = incl - nch;  // exclusive prefix
      const uint32_t starts = __reduce_or_sync(0xffffffffu, (take & lanebit) ? (1u << start) : 0u);
      // lane j < total handles child j: its entry is the number of starts at or below j, minus 1
      const int my_e = __popc(starts & (lanebit | lt_mask)) - 1;
      const int e_src = lane < total ? my_e : 0;
      const uint32_t pent = __shfl_sync(0xffffffffu, ent, e_src);
      const uint32_t pmask = __shfl_sync(0xffffffffu, emask, e_src);
      const int pstart = __shfl_sync(0xffffffffu, start, e_src);
      const bool has = lane < total;
      const int c = has ? (int)(pent & ((1u << kChildShift) - 1u)) + (lane - pstart) : 0;

      // ---- classify the child against the group's bounding box
      float4 mac = make_float4(0.f, 0.f, 0.f, 0.f);
      int4 link = make_int4(0, 0, 0, 0);
      uint32_t am = 0, om = 0;
      bool mixed = false;
      if (has) {
        mac = __ldg(&nodes[c].mac);
        link = __ldg(&nodes[c].link);
        const float s2 = fabsf(mac.w);
        const float lx = fmaxf(fmaxf(bminx - mac.x, mac.x - bmaxx), 0.f);
        const float ly = fmaxf(fmaxf(bminy - mac.y, mac.y - bmaxy), 0.f);
        const float lz = fmaxf(fmaxf(bminz - mac.z, mac.z - bmaxz), 0.f);
        const float hx = fmaxf(fabsf(mac.x - bminx), fabsf(mac.x - bmaxx));
        const float hy = fmaxf(fabsf(mac.y - bminy), fabsf(mac.y - bmaxy));
        const float hz = fmaxf(fabsf(mac.z - bminz), fabsf(mac.z - bmaxz));
        const float dmin2 = fmaf(lx, lx, fmaf(ly, ly, lz * lz));
        const float dmax2 = fmaf(hx, hx, fmaf(hy, hy, hz * hz));
        if (s2 < acc_scale * dmin2) {
          am = pmask;
        } else if (s2 >= open_scale * dmax2) {
          om = pmask;
        } else {
          mixed = true;
        }
      }
      // per-lane MAC for the mixed children, one ballot each: the mixed children's barycentres
      // and sizes are staged in shared memory (one broadcast load per child), and the child's
      // own lane applies its open mask to the ballot
      uint32_t mixed_bits = __ballot_sync(0xffffffffu, mixed);
      if (mixed_bits) {
        __syncwarp();
        if (mixed) s.st0[lane] = make_float4(mac.x, mac.y, mac.z, fabsf(mac.w));
        __syncwarp();
        do {
          const int j = __ffs(mixed_bits) - 1;
          mixed_bits &= mixed_bits - 1;
          const float4 cm = s.st0[j];
          const float dx = cm.x - p.x, dy = cm.y - p.y, dz = cm.z - p.z;
          const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const uint32_t a = __ballot_sync(0xffffffffu, cm.w < theta2 * d2);
          if (lane == j) {
            am = a & pmask;
            om = pmask & ~a;
          }
        } while (mixed_bits);
      }

      // ---- appends
      const bool single = mac.w < 0.f;  // single-body leaf
      const bool is_cell = kQuad && am != 0u && !single;
      const bool is_npt = am != 0u && !is_cell;
      const bool is_push = om != 0u && link.y > 0;
      const bool is_leaf = om != 0u && link.y == 0;

      if (kQuad) {
        const uint32_t bal = __ballot_sync(0xffffffffu, is_cell);
        if (bal) {
          __syncwarp();
          if (is_cell) {
            const int pos = ncell + __popc(bal & lt_mask);
            s.cell_node[pos] = c;
            s.cell_mask[pos] = am;
            cnt_cell += __popc(am);
          }
          ncell += __popc(bal);
          if (ncell >= 32) {
            eval_cells<kRec, Cfg::kForm>(s,32, nodes, lanebit, p.x, p.y, p.z, eps2, acc, ev_cell, rec);
            shift_down(s.cell_node, s.cell_mask, ncell, lane);
            ncell -= 32;
          }
        }
      }
      {
        const uint32_t bal = __ballot_sync(0xffffffffu, is_npt);
        if (bal) {
          __syncwarp();
          if (is_npt) {
            const int pos = npt + __popc(bal & lt_mask);
            s.pt_idx[pos] = -(c + 1);
            s.pt_mask[pos] = am;
            cnt_pt += __popc(am);
          }
          npt += __popc(bal);
          if (npt >= 32) {
            eval_points<kSelfTest, kRec>(s,32, nodes, tpos, lanebit, p.x, p.y, p.z, eps2, acc, ev_pt, rec);
            shift_down(s.pt_idx, s.pt_mask, npt, lane);
            npt -= 32;
          }
        }
      }
      {
        const uint32_t bal = __ballot_sync(0xffffffffu, is_push);
        if (bal) {
          const int np = __popc(bal);
          if (sp + np > kStack) {
            overflow = true;
            break;
          }
          __syncwarp();
          if (is_push) {
            const int pos = sp + __popc(bal & lt_mask);
            s.stk_node[pos] = (uint32_t)link.x | ((uint32_t)link.y << kChildShift);
            s.stk_mask[pos] = om;
          }
          sp += np;
        }
      }
      {
        // opened leaves: expand their bodies into the point buffer, 32 at a time
        const int cntb = is_leaf ? link.w : 0;
        int incb = cntb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, incb, o);
          if (lane >= o) incb += y;
        }
        const int totb = __shfl_sync(0xffffffffu, incb, 31);
        if (totb > 0) {
          if (is_leaf) {
            // self pairs inside this leaf: lanes of the mask whose own body is a member
            const int lo = max(link.z, gbase), hi = min(link.z + link.w, gbase + 32);
            uint32_t own = 0;
            if (hi > lo) own = (hi - lo >= 32 ? 0xffffffffu : ((1u << (hi - lo)) - 1u)) << (lo - gbase);
            cnt_pt += (long long)cntb * __popc(om) - __popc(own & om);
          }
          __syncwarp();
          s.ex_first[lane] = link.z;
          s.ex_off[lane] = incb - cntb;
          s.ex_mask[lane] = is_leaf ? om : 0u;
          __syncwarp();
          for (int base = 0; base < totb; base += 32) {
            const int gi = base + lane;
            const int kk = min(32, totb - base);
            if (gi < totb) {
              // owner: last lane whose exclusive offset is <= gi (empty lanes share offsets
              // with their successor, so the search lands on the lane that owns gi)
              int lo2 = 0, hi2 = 31;
              while (lo2 < hi2) {
                const int mid = (lo2 + hi2 + 1) >> 1;
                if (s.ex_off[mid] <= gi)
                  lo2 = mid;
                else
                  hi2 = mid - 1;
              }
              s.pt_idx[npt + lane] = s.ex_first[lo2] + (gi - s.ex_off[lo2]);
              s.pt_mask[npt + lane] = s.ex_mask[lo2];
            }
            npt += kk;
            if (npt >= 32) {
              eval_points<kSelfTest, kRec>(s,32, nodes, tpos, lanebit, p.x, p.y, p.z, eps2, acc, ev_pt, rec);
              shift_down(s.pt_idx, s.pt_mask, npt, lane);
              npt -= 32;
            }
            __syncwarp();
          }
        }
      }
    }
    if (ncell > 0) eval_cells<kRec, Cfg::kForm>(s,ncell, nodes, lanebit, p.x, p.y, p.z, eps2, acc, ev_cell, rec);
    if (npt > 0) eval_points<kSelfTest, kRec>(s,npt, nodes, tpos, lanebit, p.x, p.y, p.z, eps2, acc, ev_pt, rec);
    if (valid) {
      const uint32_t slot = __ldg(tslot + i);
      const float ax = acc.sx, ay = acc.sy, az = acc.sz;
      acc_slot[slot] = make_float4(ax, ay, az, 0.f);
      if (vel_kick) {
        float4 v = vel_kick[slot];
        v.x += ax * half_dt;
        v.y += ay * half_dt;
        v.z += az * half_dt;
        vel_kick[slot] = v;
        // a second copy of the kicked velocity (the caller's mapped pinned buffer of a host-IO
        // step: the download then rides on the walk instead of following it)
        if (vel_copy) vel_copy[slot] = v;
      }
    }
    tot_cell += (unsigned long long)cnt_cell;
    tot_pt += (unsigned long long)cnt_pt;
    if (overflow) break;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    tot_cell += __shfl_xor_sync(0xffffffffu, tot_cell, o);
    tot_pt += __shfl_xor_sync(0xffffffffu, tot_pt, o);
  }
  if (lane == 0) {
    if (overflow) atomicOr(err, kErrStack);
    if (tot_cell | tot_pt) {
      atomicAdd(&ctr->cell, tot_cell);
      atomicAdd(&ctr->p2p, tot_pt);
    }
    if (ev_cell | ev_pt) {
      atomicAdd(&ctr->cell_evals, ev_cell);
      atomicAdd(&ctr->point_evals, ev_pt);
    }
  }
}

// Persistent grid of one walk instantiation on the current device: every block that can be
// resident at once (kept per device; bh_create fills it through walk_init before any capture).
constexpr int kWalkMaxDevices = 64;
template <bool kQuad, bool kSelf, bool kRec, class Cfg>
int walk_grid() {
  static int blocks[kWalkMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kWalkMaxDevices) {
    cudaGetLastError();
    dev = 0;
  }
  if (blocks[dev] == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<kQuad, kSelf, kRec, Cfg>, Cfg::kThreads, 0);
    blocks[dev] = max(1, sms * max(1, per_sm));
  }
  return blocks[dev];
}

template <bool kQuad, bool kSelf, class Cfg = CfgDefault>
void launch_walk_t(bh_ctx* c, int n, float theta2, float eps2, float4* acc_slot, float4* vel_kick, float half_dt,
                   float4* vel_copy, bool batch, int gsize = 32) {
  const int ngroups = batch ? c->ngroups : (n + gsize - 1) / gsize;
  const int grid = min(walk_grid<kQuad, kSelf, false, Cfg>(), ngroups / Cfg::kWarps + 1);
  k_walk<kQuad, kSelf, false, Cfg><<<grid, Cfg::kThreads, 0, c->stream>>>(
      c->wnode, c->tpos, c->tslot, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch ? c->groups : nullptr,
      c->ngroups, gsize, c->counters, c->err);
}

// Launch shapes the autotuner chooses from for the quadrupole walk with positive softening
// (the benchmarked path): block size, register budget (resident blocks per SM) and stack depth.
// Static shared memory caps a block at 48 KB, which bounds warps x stack depth.
using Cfg1 = WalkCfg<8, 3, 384>;
using Cfg2 = WalkCfg<8, 2, 384>;
using Cfg3 = WalkCfg<4, 8, 384>;
using Cfg4 = WalkCfg<4, 6, 384>;
using Cfg5 = WalkCfg<4, 8, 512>;
using Cfg6 = WalkCfg<8, 4, 384, 1>;
using Cfg7 = WalkCfg<4, 8, 384, 1>;
// variants 8 and 9: the default shape with groups of 16 and 8 bodies (single systems; more,
// smaller groups fill the GPU when N is small)
// variants 10 and 11: 104 registers (two 8-warp blocks per SM) with groups of 16 and 8 bodies:
// small single systems, where a few warps per SM walk and the walk's time is one warp's chain of
// dependent latencies, which more registers let the compiler overlap
constexpr int kVariants = 12;

template <class Cfg>
WalkVariant variant_info(int group = 32) {
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_walk<true, false, false, Cfg>);
  return {Cfg::kWarps, Cfg::kMinBlocks, Cfg::kStack, Cfg::kForm, fa.numRegs, group};
}

void launch_quad_variant(bh_ctx* c, int v, int n, float theta2, float eps2, float4* acc_slot, float4* vel_kick,
                         float half_dt, float4* vel_copy, bool batch) {
  switch (v) {
    case 1: launch_walk_t<true, false, Cfg1>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch); break;
    case 2: launch_walk_t<true, false, Cfg2>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch); break;
    case 3: launch_walk_t<true, false, Cfg3>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch); break;
    case 4: launch_walk_t<true, false, Cfg4>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch); break;
    case 5: launch_walk_t<true, false, Cfg5>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch); break;
    case 6: launch_walk_t<true, false, Cfg6>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch); break;
    case 7: launch_walk_t<true, false, Cfg7>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch); break;
    case 8:
      launch_walk_t<true, false, CfgDefault>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch, 16);
      break;
    case 9:
      launch_walk_t<true, false, CfgDefault>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch, 8);
      break;
    case 10:
      launch_walk_t<true, false, Cfg2>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch, 16);
      break;
    case 11:
      launch_walk_t<true, false, Cfg2>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch, 8);
      break;
    default:
      launch_walk_t<true, false, CfgDefault>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch);
      break;
  }
}

}  // namespace

int walk_variants() { return kVariants; }

WalkVariant walk_variant_info(int v) {
  switch (v) {
    case 1: return variant_info<Cfg1>();
    case 2: return variant_info<Cfg2>();
    case 3: return variant_info<Cfg3>();
    case 4: return variant_info<Cfg4>();
    case 5: return variant_info<Cfg5>();
    case 6: return variant_info<Cfg6>();
    case 7: return variant_info<Cfg7>();
    case 8: return variant_info<CfgDefault>(16);
    case 9: return variant_info<CfgDefault>(8);
    case 10: return variant_info<Cfg2>(16);
    case 11: return variant_info<Cfg2>(8);
    default: return variant_info<CfgDefault>();
  }
}

// One force-only walk with the given variant (the autotuner's trial); acc_out by slot.
void launch_walk_variant(bh_ctx* c, int v, int n, float theta, float eps, float4* acc_out, bool batch) {
  if (n <= 0) return;
  cudaMemsetAsync(&c->counters->group_next, 0, sizeof(unsigned), c->stream);
  c->launches += 1;
  launch_quad_variant(c, v, n, theta * theta, eps * eps, acc_out, nullptr, 0.f, nullptr, batch);
}

// Occupancy queries done once per process, before any stream capture.
void walk_init() {
  walk_grid<true, true, false, CfgDefault>();
  walk_grid<true, false, false, CfgDefault>();
  walk_grid<false, true, false, CfgDefault>();
  walk_grid<false, false, false, CfgDefault>();
  walk_grid<true, false, true, CfgDefault>();
  walk_grid<true, false, false, Cfg1>();
  walk_grid<true, false, false, Cfg2>();
  walk_grid<true, false, false, Cfg3>();
  walk_grid<true, false, false, Cfg4>();
  walk_grid<true, false, false, Cfg5>();
  walk_grid<true, false, false, Cfg6>();
  walk_grid<true, false, false, Cfg7>();
}

#ifndef BH_LITERAL_MIN_GROUP
#define BH_LITERAL_MIN_GROUP 4
#endif
// smallest group of the literal walk (the app's frame, 4 444 bodies: groups of 8 / 4 / 2 walk in
// 55.1 / 50.5 / 50.5 us)
constexpr int kLiteralMinGroup = BH_LITERAL_MIN_GROUP;

void launch_walk(bh_ctx* c, int n, float theta, float eps, int mode, float4* acc_slot, float4* vel_kick,
                 float half_dt, bool batch, float4* vel_copy) {
  if (n <= 0) return;
  cudaMemsetAsync(&c->counters->group_next, 0, sizeof(unsigned), c->stream);
  c->launches += 1;
  const float theta2 = theta * theta, eps2 = eps * eps;
  const bool quad = mode == BH_MULTIPOLE_QUADRUPOLE;
  const bool self = !(eps2 > 0.f);
  if (quad) {
    if (self)
      launch_walk_t<true, true>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch);
    else
      launch_quad_variant(c, c->walk_variant, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch);
  } else {
    // the literal walk has no tuned variants: its group size follows N, the largest of 32, 16,
    // 8 and 4 bodies that still gives at least 1024 groups (about seven warps per SM; the tuned
    // quadrupole walk picks 8 at 4 444 bodies, 16 at 16 384 and 32 at 2^22)
    int gsize = 32;
    while (gsize > kLiteralMinGroup && (n + gsize - 1) / gsize < 1024) gsize /= 2;
    if (self)
      launch_walk_t<false, true>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch, gsize);
    else
      launch_walk_t<false, false>(c, n, theta2, eps2, acc_slot, vel_kick, half_dt, vel_copy, batch, gsize);
  }
}

}  // namespace bh

namespace bh {

// The walk of the differentiable path: quadrupole multipoles, positive softening, and every
// flushed interaction buffer appended to `tape` (tape_count counts chunks; overflow of tape_cap
// sets the tape error bit).
void launch_walk_record(bh_ctx* c, int n, float theta, float eps, float4* acc_slot, float4* vel_kick, float half_dt,
                        Chunk* tape, unsigned* tape_count, int tape_cap) {
  if (n <= 0) return;
  cudaMemsetAsync(&c->counters->group_next, 0, sizeof(unsigned), c->stream);
  c->launches += 1;
  const int grid = min(walk_grid<true, false, true, CfgDefault>(), ((n + 31) / 32) / kWarps + 1);
  k_walk<true, false, true><<<grid, kThreads, 0, c->stream>>>(c->wnode, c->tpos, c->tslot, n, theta * theta,
                                                              eps * eps, acc_slot, vel_kick, half_dt, nullptr,
                                                              nullptr, 0, 32, c->counters, c->err, tape, tape_count,
                                                              tape_cap);
}

}  // namespace bh
