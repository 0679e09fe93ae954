// Conservation diagnostics (bh_energy_diag): kinetic and potential energy, linear and angular
// momentum of the current state. The reference has none; these measure the drift of the
// integrator and the tree force over a run.
//
// The potential of body i is taken over the current tree with the reference's opening test
// (s^2 / d^2 < theta^2 with s the node edge and d the distance to the node's barycentre,
// src/HashedOctree.cpp:872-885) and the multipoles the tree was built with:
//   accepted node  phi -= M / D + (d.Q.d) / (2 D^5),   D^2 = |d|^2 + eps^2,  d = C - x
//   opened leaf    phi -= m_j / D for every member j at a position other than x
// (the potential whose gradient is the monopole + quadrupole force of the walk). One thread per
// body walks the tree on its own stack: this is an O(N log N) diagnostic launched a few times
// per run, not a per-step kernel. Energy sums are accumulated in FP64.
#include <cuda_runtime.h>

#include <cstring>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 128;
constexpr int kStack = 8 * (kMaxDepth + 2);  // a node pushes at most 8 children per level
constexpr int kSums = 12;  // kinetic, potential, momentum (3), angular momentum (3), mass, mass-weighted x (3)

__device__ __forceinline__ void block_add(double (&v)[kSums], double* __restrict__ out) {
  __shared__ double sh[kThreads / 32][kSums];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kSums; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < kSums) {
    double x = 0;
    for (int i = 0; i < kThreads / 32; ++i) x += sh[i][threadIdx.x];
    if (x != 0.0) atomicAdd(out + threadIdx.x, x);
  }
}

// Potential of each body (tree order i, written to its slot) and the potential energy sum.
__global__ __launch_bounds__(kThreads) void k_potential(const WalkNode* __restrict__ nodes,
                                                        const float4* __restrict__ tpos,
                                                        const uint32_t* __restrict__ tslot, int n, float theta2,
                                                        float eps2, int quad, float* __restrict__ pot_slot,
                                                        double* __restrict__ sums, uint32_t* __restrict__ err) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  double v[kSums] = {};
  if (i < n) {
    const float4 p = tpos[i];
    int stk[kStack];
    int sp = 0;
    stk[sp++] = 0;
    float phi = 0.f, comp = 0.f;  // Kahan-compensated sum
    auto add = [&](float term) {
      const float y = -term - comp;
      const float t = phi + y;
      comp = (t - phi) - y;
      phi = t;
    };
    while (sp > 0) {
      const int node = stk[--sp];
      const int4 link = nodes[node].link;
      if (link.y > 0) {
        for (int c = link.x; c < link.x + link.y; ++c) {
          const float4 mac = nodes[c].mac;
          const float dx = mac.x - p.x, dy = mac.y - p.y, dz = mac.z - p.z;
          const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const float s2 = fabsf(mac.w);
          if (s2 < theta2 * d2) {  // accepted: s^2 / d^2 < theta^2 (d2 > 0 here)
            const float4 mq = nodes[c].mq;
            const float D2 = d2 + eps2;
            const float rinv = rsqrtf(D2);
            float term = mq.x * rinv;
            if (quad && nodes[c].link.w > 1) {
              const float4 q2 = nodes[c].q2;
              const float qx = fmaf(mq.y, dx, fmaf(mq.z, dy, mq.w * dz));
              const float qy = fmaf(mq.z, dx, fmaf(q2.x, dy, q2.y * dz));
              const float qz = fmaf(mq.w, dx, fmaf(q2.y, dy, q2.z * dz));
              const float s = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
              const float r2i = rinv * rinv;
              term = fmaf(0.5f * s, rinv * r2i * r2i, term);
            }
            add(term);
          } else if (sp < kStack) {
            stk[sp++] = c;
          } else {
            atomicOr(err, kErrStack);
          }
        }
      } else {
        for (int b = link.z; b < link.z + link.w; ++b) {
          const float4 q = tpos[b];
          if (q.x == p.x && q.y == p.y && q.z == p.z) continue;  // self (and coincident) skip by position
          const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
          add(q.w * rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)))));
        }
      }
    }
    if (pot_slot) pot_slot[tslot[i]] = phi;
    v[1] = 0.5 * (double)p.w * (double)phi;
  }
  block_add(v, sums);
}

// Kinetic energy, momentum, angular momentum, mass and centre of mass over the slots.
__global__ __launch_bounds__(kThreads) void k_moments(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                      int n, double* __restrict__ sums) {
  double v[kSums] = {};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const float4 p = pos[i], u = vel[i];
    const double m = p.w, x = p.x, y = p.y, z = p.z, vx = u.x, vy = u.y, vz = u.z;
    v[0] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    v[2] += m * vx;
    v[3] += m * vy;
    v[4] += m * vz;
    v[5] += m * (y * vz - z * vy);
    v[6] += m * (z * vx - x * vz);
    v[7] += m * (x * vy - y * vx);
    v[8] += m;
    v[9] += m * x;
    v[10] += m * y;
    v[11] += m * z;
  }
  block_add(v, sums);
}

}  // namespace
}  // namespace bh

using namespace bh;

extern "C" {

bh_status bh_energy_diag(bh_ctx* c, double theta, double eps, bh_energy* out, float* pot_out) {
  bh::Range range_("bh_energy_diag");
  if (!c || !out || !(theta >= 0) || !(eps >= 0)) return BH_ERR_INVALID_ARG;
  if (!c->tree_valid) return BH_ERR_NO_TREE;
  cudaSetDevice(c->device);
  const int n = (int)c->n;
  std::memset(out, 0, sizeof(*out));
  if (n == 0) return BH_OK;
  double* sums = nullptr;
  float* pot = nullptr;
  BH_TRY(dalloc(&sums, kSums));
  if (pot_out && dalloc(&pot, (size_t)n) != BH_OK) {
    dfree(sums);
    return BH_ERR_OOM;
  }
  clear_device_flags(c);
  cudaMemsetAsync(sums, 0, sizeof(double) * kSums, c->stream);
  c->launches += 2;
  k_potential<<<(n + kThreads - 1) / kThreads, kThreads, 0, c->stream>>>(
      c->wnode, c->tpos, c->tslot, n, (float)(theta * theta), (float)(eps * eps),
      c->tree_mode == BH_MULTIPOLE_QUADRUPOLE ? 1 : 0, pot, sums, c->err);
  const int sms = c->sms;
  const int grid = (n + kThreads - 1) / kThreads < sms * 8 ? (n + kThreads - 1) / kThreads : sms * 8;
  k_moments<<<grid, kThreads, 0, c->stream>>>(c->pos[c->cur], c->vel[c->cur], n, sums);
  double h[kSums];
  cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (pot_out) cudaMemcpyAsync(pot_out, pot, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
  uint32_t e = 0;
  bh_status s = last_launch();
  if (s == BH_OK) s = sync_and_check(c, &e);
  dfree(sums);
  dfree(pot);
  BH_TRY(s);
  if (e) return err_to_status(e);
  out->kinetic = h[0];
  out->potential = h[1];
  out->total = h[0] + h[1];
  for (int a = 0; a < 3; ++a) {
    out->momentum[a] = h[2 + a];
    out->angular_momentum[a] = h[5 + a];
    out->com[a] = h[8] != 0 ? h[9 + a] / h[8] : 0.0;
  }
  out->mass = h[8];
  return BH_OK;
}

}  // extern "C"
