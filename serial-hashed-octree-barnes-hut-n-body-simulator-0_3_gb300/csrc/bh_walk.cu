// Tree walk + force: ComputeHOTOctreeForce / TraverseHOTInteractionList /
// ComputeHOTForceInteractionList / LinearHashedOctree::MAC (src/HashedOctree.hpp:262-459,
// src/HashedOctree.cpp:872-885), one warp per group of 32 consecutive bodies in tree order.
//
// Per-lane exactness. The reference walks each body separately: pop a node; test each
// existing child with the MAC size^2 / d^2 < theta^2 against the body; accepted children go
// to the body's interaction list, the others are pushed; a popped leaf is added unless it is
// the body itself (same position). Here the warp walks once for its 32 bodies and every stack
// entry carries the 32-bit mask of lanes for which the node is still open. Each child is
// tested by every lane of the mask (one broadcast load, one ballot): lanes that accept it
// record it as a multipole interaction with that lane mask, the remaining lanes open it. So
// every lane ends up with exactly the interaction set the reference builds for its body.
//
// Interactions are buffered per warp in shared memory, 32 at a time: each lane stages one
// node's data (a broadcast-free coalesced gather), then all lanes run over the buffer, and a
// lane adds an entry's term only when its bit is set in that entry's mask. Two buffers:
//   cells  : accepted nodes with more than one body — monopole + quadrupole (intended mode)
//   points : single bodies — accepted single-body leaves, members of opened leaves, and (in
//            literal mode) every accepted node as a point mass at its pseudo-barycentre.
// Points at exactly the lane's own position contribute nothing (the reference's self-skip).
// Sums are FP32 per buffer flush, added into Kahan-compensated per-lane totals.
#include <cuda_runtime.h>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kStack = 192;  // >= 7 * 21 + 8: LIFO walk keeps at most 7 pending siblings per depth
constexpr int kPtBuf = 64;

struct WarpSmem {
  int stack_node[kStack];
  unsigned stack_mask[kStack];
  int cell_node[32];
  unsigned cell_mask[32];
  int pt_idx[kPtBuf];  // >= 0: body (tree order); < 0: -(node + 1)
  unsigned pt_mask[kPtBuf];
  float4 st0[32];
  float4 st1[32];
  float4 st2[32];
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

__device__ __forceinline__ void flush_cells(WarpSmem& s, int ncell, const WalkNode* __restrict__ nodes, int lane,
                                            float px, float py, float pz, float eps2, Acc& acc, unsigned& cnt) {
  __syncwarp();
  if (lane < ncell) {
    const WalkNode* nd = nodes + s.cell_node[lane];
    s.st0[lane] = __ldg(&nd->mac);
    s.st1[lane] = __ldg(&nd->mq);
    s.st2[lane] = __ldg(&nd->q2);
  }
  __syncwarp();
  float bx = 0.f, by = 0.f, bz = 0.f;
  for (int j = 0; j < ncell; ++j) {
    const unsigned mk = s.cell_mask[j];
    const float4 c0 = s.st0[j], c1 = s.st1[j], c2 = s.st2[j];
    const float dx = c0.x - px, dy = c0.y - py, dz = c0.z - pz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    const float rinv = rsqrtf(r2);
    const float rinv2 = rinv * rinv;
    const float rinv3 = rinv * rinv2;
    const float rinv5 = rinv3 * rinv2;
    // Q.d with Q = (Qxx, Qxy, Qxz, Qyy, Qyz, Qzz) = (c1.y, c1.z, c1.w, c2.x, c2.y, c2.z)
    const float qx = fmaf(c1.y, dx, fmaf(c1.z, dy, c1.w * dz));
    const float qy = fmaf(c1.z, dx, fmaf(c2.x, dy, c2.y * dz));
    const float qz = fmaf(c1.w, dx, fmaf(c2.y, dy, c2.z * dz));
    const float qr = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
    // a += m d / D^3 - Q.d / D^5 + 2.5 (d.Q.d) d / D^7
    const float radial = fmaf(c1.x, rinv3, 2.5f * qr * rinv5 * rinv2);
    const float fx = fmaf(radial, dx, -qx * rinv5);
    const float fy = fmaf(radial, dy, -qy * rinv5);
    const float fz = fmaf(radial, dz, -qz * rinv5);
    if ((mk >> lane) & 1u) {
      bx += fx;
      by += fy;
      bz += fz;
      ++cnt;
    }
  }
  acc.add(bx, by, bz);
}

__device__ __forceinline__ void flush_points(WarpSmem& s, int npt, const WalkNode* __restrict__ nodes,
                                             const float4* __restrict__ tpos, int lane, float px, float py,
                                             float pz, float eps2, Acc& acc, unsigned& cnt) {
  __syncwarp();
  if (lane < npt) {
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
  for (int j = 0; j < npt; ++j) {
    const unsigned mk = s.pt_mask[j];
    const float4 v = s.st0[j];
    const float dx = v.x - px, dy = v.y - py, dz = v.z - pz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    const float rinv = rsqrtf(r2);
    const float mr3 = v.w * rinv * rinv * rinv;
    const bool self = (dx == 0.f) & (dy == 0.f) & (dz == 0.f);
    if (((mk >> lane) & 1u) && !self) {
      bx = fmaf(mr3, dx, bx);
      by = fmaf(mr3, dy, by);
      bz = fmaf(mr3, dz, bz);
      ++cnt;
    }
  }
  acc.add(bx, by, bz);
}

template <bool kQuad>
__global__ __launch_bounds__(kThreads) void k_walk(const WalkNode* __restrict__ nodes,
                                                   const float4* __restrict__ tpos,
                                                   const uint32_t* __restrict__ tslot, int n, float theta2,
                                                   float eps2, float4* __restrict__ acc_slot,
                                                   float4* __restrict__ vel_kick, float half_dt,
                                                   Counters* __restrict__ ctr, uint32_t* __restrict__ err) {
  __shared__ WarpSmem smem[kWarps];
  const int lane = threadIdx.x & 31;
  WarpSmem& s = smem[threadIdx.x >> 5];
  if (*((volatile uint32_t*)err) & (kErrNodes | kErrTimeout)) return;
  const int ngroups = (n + 31) >> 5;
  const int4 root_link = __ldg(&nodes[0].link);
  unsigned long long tot_cell = 0, tot_pt = 0;

  for (;;) {
    int g = 0;
    if (lane == 0) g = (int)atomicAdd(&ctr->group_next, 1u);
    g = __shfl_sync(0xffffffffu, g, 0);
    if (g >= ngroups) break;
    const int i = g * 32 + lane;
    const bool valid = i < n;
    const float4 p = valid ? __ldg(tpos + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    Acc acc;
    unsigned cnt_cell = 0, cnt_pt = 0;
    int sp = 0, ncell = 0, npt = 0;
    bool overflow = false;

    auto append_points = [&](int first, int count, unsigned mask) {
      for (int off = 0; off < count; off += 32) {
        const int k = min(32, count - off);
        __syncwarp();
        if (lane < k) {
          s.pt_idx[npt + lane] = first + off + lane;
          s.pt_mask[npt + lane] = mask;
        }
        npt += k;
        if (npt >= 32) {
          flush_points(s, 32, nodes, tpos, lane, p.x, p.y, p.z, eps2, acc, cnt_pt);
          __syncwarp();
          const int rest = npt - 32;
          if (lane < rest) {
            const int e = s.pt_idx[32 + lane];
            const unsigned m = s.pt_mask[32 + lane];
            __syncwarp(__activemask());
            s.pt_idx[lane] = e;
            s.pt_mask[lane] = m;
          }
          npt = rest;
        }
      }
    };

    if (root_link.y == 0) {
      append_points(root_link.z, root_link.w, active);
    } else {
      if (lane == 0) {
        s.stack_node[0] = 0;
        s.stack_mask[0] = active;
      }
      sp = 1;
    }
    while (sp > 0) {
      --sp;
      __syncwarp();
      const int nd = s.stack_node[sp];
      const unsigned m = s.stack_mask[sp];
      const int4 link = __ldg(&nodes[nd].link);
      for (int c = link.x; c < link.x + link.y; ++c) {
        const float4 mac = __ldg(&nodes[c].mac);
        const float dx = mac.x - p.x, dy = mac.y - p.y, dz = mac.z - p.z;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool accept = fabsf(mac.w) < theta2 * d2;
        const unsigned am = __ballot_sync(0xffffffffu, accept) & m;
        const unsigned om = m & ~am;
        if (am) {
          if (!kQuad || mac.w < 0.f) {
            __syncwarp();
            if (lane == 0) {
              s.pt_idx[npt] = -(c + 1);
              s.pt_mask[npt] = am;
            }
            ++npt;
            if (npt >= 32) {
              flush_points(s, 32, nodes, tpos, lane, p.x, p.y, p.z, eps2, acc, cnt_pt);
              npt = 0;
            }
          } else {
            __syncwarp();
            if (lane == 0) {
              s.cell_node[ncell] = c;
              s.cell_mask[ncell] = am;
            }
            ++ncell;
            if (ncell == 32) {
              flush_cells(s, 32, nodes, lane, p.x, p.y, p.z, eps2, acc, cnt_cell);
              ncell = 0;
            }
          }
        }
        if (om) {
          const int4 cl = __ldg(&nodes[c].link);
          if (cl.y > 0) {
            if (sp >= kStack) {
              overflow = true;
              break;
            }
            __syncwarp();
            if (lane == 0) {
              s.stack_node[sp] = c;
              s.stack_mask[sp] = om;
            }
            ++sp;
          } else {
            append_points(cl.z, cl.w, om);
          }
        }
      }
      if (overflow) break;
    }
    if (ncell > 0) flush_cells(s, ncell, nodes, lane, p.x, p.y, p.z, eps2, acc, cnt_cell);
    if (npt > 0) flush_points(s, npt, nodes, tpos, lane, p.x, p.y, p.z, eps2, acc, cnt_pt);
    if (overflow && lane == 0) atomicOr(err, kErrStack);
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
      }
      tot_cell += cnt_cell;
      tot_pt += cnt_pt;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    tot_cell += __shfl_down_sync(0xffffffffu, tot_cell, o);
    tot_pt += __shfl_down_sync(0xffffffffu, tot_pt, o);
  }
  if (lane == 0 && (tot_cell | tot_pt)) {
    atomicAdd(&ctr->cell, tot_cell);
    atomicAdd(&ctr->p2p, tot_pt);
  }
}

int walk_grid(bool quad) {
  static int blocks[2] = {0, 0};
  int& b = blocks[quad ? 1 : 0];
  if (b == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (quad)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<true>, kThreads, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<false>, kThreads, 0);
    b = max(1, sms * max(1, per_sm));
  }
  return b;
}

}  // namespace

void launch_walk(bh_ctx* c, int n, float theta, float eps, int mode, float4* acc_slot, float4* vel_kick,
                 float half_dt) {
  if (n <= 0) return;
  cudaMemsetAsync(&c->counters->group_next, 0, sizeof(unsigned), c->stream);
  const float theta2 = theta * theta, eps2 = eps * eps;
  const bool quad = mode == BH_MULTIPOLE_QUADRUPOLE;
  const int grid = min(walk_grid(quad), (n + 31) / 32 / kWarps + 1);
  c->launches += 1;
  if (quad)
    k_walk<true><<<grid, kThreads, 0, c->stream>>>(c->wnode, c->tpos, c->tslot, n, theta2, eps2, acc_slot,
                                                   vel_kick, half_dt, c->counters, c->err);
  else
    k_walk<false><<<grid, kThreads, 0, c->stream>>>(c->wnode, c->tpos, c->tslot, n, theta2, eps2, acc_slot,
                                                    vel_kick, half_dt, c->counters, c->err);
}

}  // namespace bh
