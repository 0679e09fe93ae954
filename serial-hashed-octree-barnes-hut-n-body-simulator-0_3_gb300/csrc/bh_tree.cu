// Bounds, Morton keys, tree keys, gathers, leapfrog halves, node discovery, upsweep and the
// node hash table.
//
// FP64 arithmetic that must reproduce the reference bit for bit uses the explicitly rounded
// intrinsics (__dadd_rn, __dmul_rn, ...), so the compiler cannot contract it into FMAs.
#include <cuda_runtime.h>

#include <algorithm>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------------------
// exact-arithmetic helpers
// ---------------------------------------------------------------------------------------

// Magic-bit spread of src/MortonKeys.hpp:100-104 with the masks of :51-58, on the full 64-bit
// word (high garbage bits of wrapped coordinates behave as in the reference).
__device__ __forceinline__ uint64_t spread_bits(uint64_t v) {
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

// Float-float arithmetic (a value is hi + lo): TwoSum (Knuth), FMA-based TwoProduct and a
// Newton-corrected quotient (Dekker 1971). About 44 significant bits from FP32 operations.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_norm(float s, float e) {
  const float hi = s + e;
  return {hi, e - (hi - s)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  return ff_norm(s, e);
}
__device__ __forceinline__ FF ff_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ FF ff_div(FF n, FF d) {
  const float q = n.hi / d.hi;
  const float p = q * d.hi;
  const float pe = fmaf(q, d.hi, -p);
  const float r = (((n.hi - p) - pe) + fmaf(-q, d.lo, n.lo)) / d.hi;
  return ff_norm(q, r);
}
// Splits a double into a float-float pair (hi = nearest float, lo = nearest float of the rest):
// the pair matches the double to about 2^-48 relative.
__device__ __forceinline__ void ff_split(double x, float& hi, float& lo) {
  hi = __double2float_rn(x);
  lo = __double2float_rn(__dsub_rn(x, (double)hi));
}

// x ~ n + f from a float-float value: n = nearest integer of hi (exactly representable), f the
// signed remainder (|f| <= 0.5 + |lo|), accurate to the pair's own error.
__device__ __forceinline__ void ff_int_frac(FF x, float& n, float& f) {
  n = rintf(x.hi);
  f = (x.hi - n) + x.lo;
}

// The reference's (spatialKey)(double) cast (src/MortonKeys.hpp:162-164) as x86-64 code
// generated by gcc evaluates it: below 2^63 (or NaN) a signed truncation, 0x8000000000000000
// when that is out of range; otherwise a truncation of x - 2^63 with bit 63 flipped.
__device__ __forceinline__ uint64_t x86_trunc_u64(double x) {
  if (!(x >= 0x1p63)) {
    if (x >= -0x1p63) return (uint64_t)__double2ll_rz(x);
    return 0x8000000000000000ull;
  }
  double y = __dsub_rn(x, 0x1p63);
  if (y < 0x1p63) return (uint64_t)__double2ll_rz(y) ^ 0x8000000000000000ull;
  return 0ull;
}

// One axis of computeMortonKey (src/MortonKeys.hpp:137-181) in the reference's own FP64
// arithmetic: (p + S) * frac, then the cast.
__device__ __noinline__ uint64_t morton_coord_exact(float x, double S, double frac) {
  return x86_trunc_u64(__dmul_rn(__dadd_rn((double)x, S), frac));
}

// The same axis with an FP32 fast path. v = (p + S) * frac is formed in float-float: for
// |v| < 2^22 the pair is within 2^-23 of the exact v, and the reference's two FP64 roundings put
// its value within |v| 2^-52 <= 2^-30 of it. When the pair lies farther than 2^-21 from every
// integer, both therefore truncate to the same integer, which the fast path returns (as the
// 64-bit two's-complement word the cast produces for |v| < 2^63). Otherwise (near an integer,
// |v| >= 2^22, or not finite) the FP64 path decides.
__device__ __forceinline__ uint64_t morton_coord(float x, const Geom& g) {
  const FF v = ff_mul(ff_add({x, 0.f}, {g.size_hi, g.size_lo}), {g.frac_hi, g.frac_lo});
  float n, f;
  ff_int_frac(v, n, f);
  if (fabsf(v.hi) < 0x1p22f && fabsf(f) > 0x1p-21f) {
    const bool pos = n > 0.f || (n == 0.f && f > 0.f);
    // truncation toward zero: floor for positive v, ceiling for negative v
    const float q = pos ? (f < 0.f ? n - 1.f : n) : (f > 0.f ? n + 1.f : n);
    return (uint64_t)(long long)q;
  }
  return morton_coord_exact(x, g.size, g.frac);
}

// computeMortonKey: the three axes interleaved x<<2 | y<<1 | z with bit 63 set
// (interleaveBits, src/MortonKeys.hpp:95-124).
__device__ __forceinline__ uint64_t morton_key(float4 p, const Geom& g) {
  const uint64_t wx = morton_coord(p.x, g), wy = morton_coord(p.y, g), wz = morton_coord(p.z, g);
  return (1ull << 63) | (spread_bits(wx) << 2) | (spread_bits(wy) << 1) | spread_bits(wz);
}

// 21-bit octant path of one coordinate below a root of centre c0 and edge E, exactly as the
// reference's descent computes it: at each depth compare p > c (DetermineOctant,
// src/OctantUtils.hpp:64-70), halve the size and move the centre by (+-0.5) * size
// (HOTNode child constructor, src/HashedNode.cpp:52-56), one FP64 rounding per level.
__device__ __noinline__ uint32_t tree_path_exact(double p, double c0, double E) {
  double c = c0, s = E;
  uint32_t k = 0;
  for (int d = 0; d < kMaxDepth; ++d) {
    uint32_t b = p > c ? 1u : 0u;
    k = (k << 1) | b;
    s = __dmul_rn(s, 0.5);
    c = __dadd_rn(c, __dmul_rn(b ? 0.5 : -0.5, s));
  }
  return k;
}

// Same path from one scaled coordinate. In exact arithmetic the level-d comparison points
// are the integers of [1, 2^21 - 1] in the units u = (p - c0) * 2^21 / E + 2^20, and the
// strict '>' makes the path ceil(u) - 1 clamped to [0, 2^21 - 1]. The reference's rounded
// centres differ from the exact ones by at most 21 half-ulps: below 2^-26 * (1 + |c0| / E) key
// units. u is formed in float-float (the splits of c0 and 2^21 / E and the pair arithmetic add
// below 2^-24 * (1 + |c0| / E)). Whenever u lies closer than the margin
// (2^-20 * (1 + |c0| / E)) to a comparison point, or is not finite, the exact recurrence
// decides instead.
__device__ __forceinline__ uint32_t tree_path(float p, int a, const Geom& g) {
  const FF d = ff_add({p, 0.f}, {-g.tc_hi[a], -g.tc_lo[a]});
  const FF u = ff_add(ff_mul(d, {g.tscale_hi, g.tscale_lo}), {1048576.f, 0.f});
  float n, f;
  ff_int_frac(u, n, f);
  float dist;
  uint32_t path;
  if (n < 1.f || (n == 1.f && f < 0.f)) {  // u < 1
    dist = (1.f - n) - f;
    path = 0u;
  } else if (n > 2097151.f || (n == 2097151.f && f > 0.f)) {  // u > 2^21 - 1
    dist = (n - 2097151.f) + f;
    path = 2097151u;
  } else {
    dist = fabsf(f);
    path = (uint32_t)(f < 0.f ? n - 1.f : n);
  }
  if (dist > g.tmargin_f) return path;  // false for NaN
  return tree_path_exact((double)p, g.tc[a], g.tedge);
}

__device__ __forceinline__ uint64_t tree_key(float4 p, const Geom& g) {
  const uint32_t kx = tree_path(p.x, 0, g), ky = tree_path(p.y, 1, g), kz = tree_path(p.z, 2, g);
  return (1ull << 63) | (spread_bits(kx) << 2) | (spread_bits(ky) << 1) | spread_bits(kz);
}

__device__ __forceinline__ void fill_tree_geom(Geom& g, const double tc[3], double tedge) {
  g.tc[0] = tc[0];
  g.tc[1] = tc[1];
  g.tc[2] = tc[2];
  g.tedge = tedge;
  g.tscale = __ddiv_rn(2097152.0, tedge);
  double cm = fmax(fabs(tc[0]), fmax(fabs(tc[1]), fabs(tc[2])));
  g.tmargin = 0x1p-20 * (1.0 + cm / tedge);
  // float-float copies for the key fast paths (size and frac are set by every caller first)
  ff_split(g.size, g.size_hi, g.size_lo);
  ff_split(g.frac, g.frac_hi, g.frac_lo);
  for (int a = 0; a < 3; ++a) ff_split(tc[a], g.tc_hi[a], g.tc_lo[a]);
  ff_split(g.tscale, g.tscale_hi, g.tscale_lo);
  g.tmargin_f = __double2float_rn(g.tmargin);
}

// ---------------------------------------------------------------------------------------
// bounds (OctantBounds(Body*, N), src/OctantUtils.cpp:27-59)
// ---------------------------------------------------------------------------------------

// Per block: FP64 sums of x, y, z (each thread strides through the bodies in a fixed order,
// then a fixed-shape tree reduction) and FP32 maxima of |x|, |y|, |z|.
__global__ __launch_bounds__(kThreads) void k_bounds_partial(const float4* __restrict__ pos, int n,
                                                             double* __restrict__ partial) {
  double sx = 0, sy = 0, sz = 0;
  float mx = 0.f, my = 0.f, mz = 0.f;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    float4 p = pos[i];
    sx = __dadd_rn(sx, (double)p.x);
    sy = __dadd_rn(sy, (double)p.y);
    sz = __dadd_rn(sz, (double)p.z);
    mx = fmaxf(mx, fabsf(p.x));
    my = fmaxf(my, fabsf(p.y));
    mz = fmaxf(mz, fabsf(p.z));
  }
  __shared__ double sh[6][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sx = __dadd_rn(sx, __shfl_down_sync(0xffffffffu, sx, o));
    sy = __dadd_rn(sy, __shfl_down_sync(0xffffffffu, sy, o));
    sz = __dadd_rn(sz, __shfl_down_sync(0xffffffffu, sz, o));
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    my = fmaxf(my, __shfl_down_sync(0xffffffffu, my, o));
    mz = fmaxf(mz, __shfl_down_sync(0xffffffffu, mz, o));
  }
  if (lane == 0) {
    sh[0][w] = sx;
    sh[1][w] = sy;
    sh[2][w] = sz;
    sh[3][w] = mx;
    sh[4][w] = my;
    sh[5][w] = mz;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double acc = sh[threadIdx.x][0];
    for (int i = 1; i < kThreads / 32; ++i)
      acc = threadIdx.x < 3 ? __dadd_rn(acc, sh[threadIdx.x][i]) : fmax(acc, sh[threadIdx.x][i]);
    partial[blockIdx.x * 6 + threadIdx.x] = acc;
  }
}

// Combines the partials (one warp: lane l sums partials l, l + 32, ... in order, then a fixed
// shuffle tree; deterministic, and only ~15 dependent FP64 additions deep): centre = sum *
// (1 / N) (Vec3D::operator/=, src/MathUtils.cpp:81-90), size = max(0, max_a (max_i |p_ia| -
// c_a)). fl(|p| - c) is monotone in |p|, so the maximum over bodies of the rounded differences
// equals the rounded difference of the maximum.
__global__ void k_bounds_final(const double* __restrict__ partial, int blocks, int n, double edge_factor,
                               Geom* __restrict__ g) {
  const int lane = threadIdx.x;
  double s[3] = {0, 0, 0}, m[3] = {0, 0, 0};
  for (int b = lane; b < blocks; b += 32)
    for (int a = 0; a < 3; ++a) {
      s[a] = __dadd_rn(s[a], partial[b * 6 + a]);
      m[a] = fmax(m[a], partial[b * 6 + 3 + a]);
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    for (int a = 0; a < 3; ++a) {
      s[a] = __dadd_rn(s[a], __shfl_down_sync(0xffffffffu, s[a], o));
      m[a] = fmax(m[a], __shfl_down_sync(0xffffffffu, m[a], o));
    }
  if (lane != 0) return;
  double c[3] = {s[0], s[1], s[2]};
  double nn = (double)n;
  if (nn != 0) {
    double inv = __ddiv_rn(1.0, nn);
    for (int a = 0; a < 3; ++a) c[a] = __dmul_rn(c[a], inv);
  }
  double S = 0;
  for (int a = 0; a < 3; ++a) {
    double v = __dsub_rn(m[a], c[a]);
    if (v > S) S = v;
  }
  for (int a = 0; a < 3; ++a) g->center[a] = c[a];
  g->size = S;
  g->frac = __ddiv_rn(2097152.0, __dmul_rn(2.0, S));
  fill_tree_geom(*g, c, __dmul_rn(S, edge_factor));
}

__global__ void k_set_geom(Geom* __restrict__ g, double c0, double c1, double c2, double S, double t0, double t1,
                           double t2, double tedge) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  g->center[0] = c0;
  g->center[1] = c1;
  g->center[2] = c2;
  g->size = S;
  g->frac = __ddiv_rn(2097152.0, __dmul_rn(2.0, S));
  double tc[3] = {t0, t1, t2};
  fill_tree_geom(*g, tc, tedge);
}

// ---------------------------------------------------------------------------------------
// keys, gathers, leapfrog
// ---------------------------------------------------------------------------------------

// body_sys (optional): system of each body; each system then uses its own geometry
// sys_geom[body_sys[i]] (batched ensembles), otherwise the single geometry *g.
__global__ __launch_bounds__(kThreads) void k_morton(const float4* __restrict__ pos, int n,
                                                     const Geom* __restrict__ g, const uint16_t* __restrict__ body_sys,
                                                     uint64_t* __restrict__ keys, uint32_t* __restrict__ idx) {
  int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Geom& gg = body_sys ? g[body_sys[i]] : *g;
  keys[i] = morton_key(pos[i], gg);
  idx[i] = (uint32_t)i;
}

// decodeMortonKey (src/MortonKeys.hpp:204-228): each axis's 21 bits de-interleaved, then
// x_int / 2^21 * 2 * S - S (the division and doubling are exact; one rounding each for the
// product and the difference, as in the reference's FP64 expression).
__global__ __launch_bounds__(kThreads) void k_decode_morton(const uint64_t* __restrict__ keys, int n, double S,
                                                            double* __restrict__ pos3) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = keys[i];
  uint32_t q[3] = {0u, 0u, 0u};
#pragma unroll
  for (int b = 0; b < kMaxDepth; ++b)
#pragma unroll
    for (int a = 0; a < 3; ++a) q[a] |= (uint32_t)((k >> (3 * b + 2 - a)) & 1ull) << b;
#pragma unroll
  for (int a = 0; a < 3; ++a) pos3[3 * i + a] = __dsub_rn(__dmul_rn((double)q[a] * 0x1p-20, S), S);
}

__global__ __launch_bounds__(kThreads) void k_treekey(const float4* __restrict__ pos, int n,
                                                      const Geom* __restrict__ g, uint64_t* __restrict__ tkeys,
                                                      uint32_t* __restrict__ tidx) {
  int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  tkeys[i] = tree_key(pos[i], *g);
  tidx[i] = (uint32_t)i;
}

__global__ __launch_bounds__(kThreads) void k_gather(const uint32_t* __restrict__ perm, int n,
                                                     const float4* __restrict__ pin, const float4* __restrict__ vin,
                                                     float4* __restrict__ pout, float4* __restrict__ vout) {
  int j = blockIdx.x * kThreads + threadIdx.x;
  if (j >= n) return;
  uint32_t i = perm[j];
  pout[j] = pin[i];
  vout[j] = vin[i];
}

// Gather into the new (Morton) order fused with the first half-kick and the drift
// (ComputePositionAtHalfTimeStep, src/Body.hpp:306-313) and with the tree key of the drifted
// position.
__global__ __launch_bounds__(kThreads) void k_gather_kd_treekey(
    const uint32_t* __restrict__ perm, int n, const float4* __restrict__ pin, const float4* __restrict__ vin,
    const float4* __restrict__ acc, int acc_follows_body, float dt, float half_dt, const Geom* __restrict__ g,
    const uint16_t* __restrict__ body_sys, float4* __restrict__ pout, float4* __restrict__ vout,
    uint64_t* __restrict__ tkeys, uint32_t* __restrict__ tidx) {
  int j = blockIdx.x * kThreads + threadIdx.x;
  if (j >= n) return;
  const uint32_t i = perm ? perm[j] : (uint32_t)j;  // no permutation: bodies keep their order
  float4 p = pin[i], v = vin[i], a = acc[acc_follows_body ? i : (uint32_t)j];
  v.x += a.x * half_dt;
  v.y += a.y * half_dt;
  v.z += a.z * half_dt;
  p.x += v.x * dt;
  p.y += v.y * dt;
  p.z += v.z * dt;
  pout[j] = p;
  vout[j] = v;
  // the sort keeps every system in its body range, so slot j's system is body_sys[j]
  tkeys[j] = tree_key(p, body_sys ? g[body_sys[j]] : *g);
  tidx[j] = (uint32_t)j;
}

__global__ __launch_bounds__(kThreads) void k_kick_drift(float4* __restrict__ pos, float4* __restrict__ vel,
                                                         const float4* __restrict__ acc, int n, float dt,
                                                         float half_dt, int drift) {
  int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  float4 v = vel[i], a = acc[i];
  v.x += a.x * half_dt;
  v.y += a.y * half_dt;
  v.z += a.z * half_dt;
  vel[i] = v;
  if (drift) {
    float4 p = pos[i];
    p.x += v.x * dt;
    p.y += v.y * dt;
    p.z += v.z * dt;
    pos[i] = p;
  }
}

__global__ __launch_bounds__(kThreads) void k_gather_tree(const uint32_t* __restrict__ tslot, int n,
                                                          const float4* __restrict__ pos,
                                                          float4* __restrict__ tpos) {
  int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  tpos[i] = pos[tslot[i]];
}

// ---------------------------------------------------------------------------------------
// node discovery
// ---------------------------------------------------------------------------------------
// The node set equals the reference's insertion result: the root, plus every prefix K of a
// body's depth-21 path whose parent holds more than leaf_cap bodies (for leaf capacity 1:
// count(parent) >= 2). Bodies are sorted by path, so every node is a contiguous body range.
// Two builds produce the same records: the all-depths build further down (single systems with
// leaf capacity up to 64), and this level build (ensembles, larger leaf capacities).
// One launch per depth turns the internal nodes of depth d into the node records of depth
// d+1, appended in key order: children get contiguous indices, depths are stored level by
// level (breadth-first), and a decoupled look-back over 256-node tiles assigns the indices.

__global__ void k_tree_init(int n, uint64_t* __restrict__ nkey, int2* __restrict__ nrange,
                            int* __restrict__ level_bounds, uint32_t* __restrict__ level_tile_ctr) {
  int t = threadIdx.x;
  if (t < kLevels) level_tile_ctr[t] = 0;
  if (t <= kLevels + 1) level_bounds[t] = (t == 0) ? 0 : (t == 1 ? (n > 0 ? 1 : 0) : -1);
  if (t == 0 && n > 0) {
    nkey[0] = 1ull;
    nrange[0] = make_int2(0, n);
  }
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
constexpr uint32_t kLbAgg = 1u << 30, kLbPrefix = 2u << 30, kLbMask = (1u << 30) - 1;
constexpr int kLbSpin = 1 << 22;

// K independent binary searches in the sorted child digits of one node: search j finds, inside
// [bnd[2Hj], bnd[2H(j+1)]), the first index whose digit is >= 2Hj + H, and stores it there.
template <int K, int H>
__device__ __forceinline__ void split_search(const uint64_t* __restrict__ tkey, int shift, int (&bnd)[9]) {
  int a[K], b[K];
#pragma unroll
  for (int j = 0; j < K; ++j) {
    a[j] = bnd[2 * H * j];
    b[j] = bnd[2 * H * (j + 1)];
  }
  for (;;) {
    bool any = false;
#pragma unroll
    for (int j = 0; j < K; ++j) any |= a[j] < b[j];
    if (!any) break;
    int dig[K];
#pragma unroll
    for (int j = 0; j < K; ++j)  // loads first, so the K searches wait on the memory together
      dig[j] = a[j] < b[j] ? (int)((tkey[(a[j] + b[j]) >> 1] >> shift) & 7ull) : 0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (a[j] >= b[j]) continue;
      const int m = (a[j] + b[j]) >> 1;
      if (dig[j] < 2 * H * j + H)
        a[j] = m + 1;
      else
        b[j] = m;
    }
  }
#pragma unroll
  for (int j = 0; j < K; ++j) bnd[2 * H * j + H] = a[j];
}

// Decoupled look-back over the tiles of one level (one thread): publishes the tile's child
// count, sums the predecessors' counts back to the first inclusive prefix (eight predecessor
// words per round trip, independent loads in flight together), publishes its own inclusive
// prefix and returns the exclusive one. Waits are bounded; on expiry the timeout bit is set.
__device__ uint32_t tile_lookback(uint32_t* __restrict__ lb, int tile, uint32_t btotal, uint32_t* __restrict__ err) {
  uint32_t* mine = lb + tile;
  st_relaxed(mine, (tile == 0 ? kLbPrefix : kLbAgg) | btotal);
  uint32_t excl = 0;
  if (tile == 0) return 0;
  constexpr int kWin = 8;
  int k = tile - 1, spins = 0;
  while (k >= 0) {
    uint32_t v[kWin];
#pragma unroll
    for (int q = 0; q < kWin; ++q)  // tile 0 always holds a prefix, so k - q < 0 is never consumed
      v[q] = (k - q >= 0) ? ld_relaxed(lb + (k - q)) : kLbPrefix;
    int used = 0;
    bool done = false;
#pragma unroll
    for (int q = 0; q < kWin; ++q) {
      if (done || used < q) continue;  // stop at a prefix or at the first unpublished tile
      const uint32_t f = v[q] & ~kLbMask;
      if (f == 0) continue;
      excl += v[q] & kLbMask;
      used = q + 1;
      done = f == kLbPrefix;
    }
    if (done) break;
    k -= used;
    if (used == 0) {
      if (++spins > kLbSpin) {
        atomicOr(err, kErrTimeout);
        break;
      }
      __nanosleep(32);
    }
  }
  st_relaxed(mine, kLbPrefix | ((excl + btotal) & kLbMask));
  return excl;
}

// The eight child ranges of one node by the whole warp: lanes 4(v-1) .. 4(v-1)+3 search for the
// first index of [lo, hi) whose child digit is >= v (v = 1..7) with four probes per round, so
// each round shrinks the interval about fivefold and the seven searches run together (about
// log5 of the range in dependent loads instead of seven binary searches). Invariant per
// search: every index below a has a smaller digit, and b is the answer or hi.
__device__ __forceinline__ void warp_child_bounds(const uint64_t* __restrict__ tkey, int shift, int lo, int hi,
                                                  int lane, int (&bnd)[9]) {
  const int g = lane >> 2, k = lane & 3, v = g + 1;
  const bool searcher = g < 7;
  int a = lo, b = hi;
  for (int it = 0; it < 40; ++it) {  // 40 rounds cover any 31-bit range
    const bool big = searcher && (b - a > 4);
    if (!__any_sync(0xffffffffu, big)) break;
    const int step = (b - a) / 5;
    bool ge = false;
    if (big) ge = (int)((tkey[a + (k + 1) * step] >> shift) & 7ull) >= v;
    const uint32_t grp = (__ballot_sync(0xffffffffu, ge) >> (4 * g)) & 0xFu;
    if (big) {
      if (grp) {
        const int f = __ffs(grp) - 1;
        b = a + (f + 1) * step;
        if (f > 0) a = a + f * step + 1;
      } else {
        a = a + 4 * step + 1;
      }
    }
  }
  const bool probe = searcher && (a + k < b);
  const bool ge = probe && (int)((tkey[a + k] >> shift) & 7ull) >= v;
  const uint32_t grp = (__ballot_sync(0xffffffffu, ge) >> (4 * g)) & 0xFu;
  const int ans = grp ? a + __ffs(grp) - 1 : b;
  bnd[0] = lo;
  bnd[8] = hi;
#pragma unroll
  for (int u = 1; u < 8; ++u) bnd[u] = __shfl_sync(0xffffffffu, ans, 4 * (u - 1));
}

__global__ __launch_bounds__(kThreads) void k_level(int d, const uint64_t* __restrict__ tkey, int leaf_cap,
                                                    uint64_t* __restrict__ nkey, int2* __restrict__ nrange,
                                                    WalkNode* __restrict__ wn, uint8_t* __restrict__ childbyte,
                                                    int* __restrict__ level_bounds,
                                                    uint32_t* __restrict__ tile_ctr, uint32_t* __restrict__ lb,
                                                    long long node_cap, uint32_t* __restrict__ err) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[kThreads / 32];
  __shared__ uint32_t s_excl;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int lo = level_bounds[d], hi = level_bounds[d + 1];
  const int count = hi - lo;
  if (count <= 0) {
    if (blockIdx.x == 0 && t == 0) level_bounds[d + 2] = hi < 0 ? -1 : hi;
    return;
  }
  if (*((volatile uint32_t*)err) & kErrNodes) {
    if (blockIdx.x == 0 && t == 0) level_bounds[d + 2] = hi;
    return;
  }
  const int shift = 3 * (kMaxDepth - 1 - d);
  if (count <= kLevelWarpNodes) {
    // few nodes with long body ranges (the top levels): one warp per node, tiles of one node
    // per warp, the child ranges found by the warp-cooperative search
    constexpr int kW = kThreads / 32;
    const int ntiles_w = (count + kW - 1) / kW;
    for (;;) {
      if (t == 0) s_tile = atomicAdd(&tile_ctr[d], 1u);
      __syncthreads();
      const int tile = (int)s_tile;
      __syncthreads();
      if (tile >= ntiles_w) break;
      const int node = lo + tile * kW + w;
      const bool valid = node < hi;  // warp-uniform
      int2 r = make_int2(0, 0);
      bool internal = false;
      int bnd[9];
      int nc = 0;
      uint32_t mask = 0;
      if (valid) {
        r = nrange[node];
        internal = r.y > leaf_cap && d < kMaxDepth;
        if (internal) {
          warp_child_bounds(tkey, shift, r.x, r.x + r.y, lane, bnd);
          for (int v = 0; v < 8; ++v)
            if (bnd[v + 1] > bnd[v]) {
              ++nc;
              mask |= 1u << v;
            }
        }
      }
      if (lane == 0) s_warp[w] = (uint32_t)nc;
      __syncthreads();
      uint32_t wadd = 0, btotal = 0;
      for (int i = 0; i < kW; ++i) {
        if (i < w) wadd += s_warp[i];
        btotal += s_warp[i];
      }
      if (t == 0) {
        const uint32_t excl = tile_lookback(lb, tile, btotal, err);
        s_excl = excl;
        if (tile == ntiles_w - 1) level_bounds[d + 2] = hi + (int)(excl + btotal);
      }
      __syncthreads();
      const long long child_base = (long long)hi + s_excl + wadd;
      if (valid) {
        const bool fits = child_base + nc <= node_cap;
        if (!fits && lane == 0) atomicOr(err, kErrNodes);
        const bool make = internal && fits;
        if (make && lane < 8 && ((mask >> lane) & 1u)) {  // lane v writes child v
          const int ci = (int)child_base + __popc(mask & ((1u << lane) - 1u));
          nkey[ci] = (nkey[node] << 3) | (uint64_t)lane;
          nrange[ci] = make_int2(bnd[lane], bnd[lane + 1] - bnd[lane]);
        }
        if (lane == 0) {
          wn[node].link = make_int4(make ? (int)child_base : -1, make ? nc : 0, r.x, r.y);
          childbyte[node] = (uint8_t)(make ? mask : 0u);
        }
      }
      __syncthreads();
    }
    return;
  }
  const int ntiles = (count + kThreads - 1) / kThreads;
  for (;;) {
    if (t == 0) s_tile = atomicAdd(&tile_ctr[d], 1u);
    __syncthreads();
    const int tile = (int)s_tile;
    __syncthreads();
    if (tile >= ntiles) break;
    const int node = lo + tile * kThreads + t;
    const bool valid = node < hi;
    int2 r = make_int2(0, 0);
    int bnd[9];
    int nc = 0;
    uint32_t mask = 0;
    bool internal = false;
    if (valid) {
      r = nrange[node];
      internal = r.y > leaf_cap && d < kMaxDepth;
      if (internal) {
        // the first index with child digit >= v, for v = 4, then 2 and 6, then 1, 3, 5, 7: each
        // round searches inside the intervals the previous round split off, and its searches are
        // independent, so their loads overlap (three dependent search depths instead of seven)
        bnd[0] = r.x;
        bnd[8] = r.x + r.y;
        split_search<1, 4>(tkey, shift, bnd);
        split_search<2, 2>(tkey, shift, bnd);
        split_search<4, 1>(tkey, shift, bnd);
        for (int v = 0; v < 8; ++v)
          if (bnd[v + 1] > bnd[v]) {
            ++nc;
            mask |= 1u << v;
          }
      }
    }
    // block exclusive scan of child counts
    uint32_t x = (uint32_t)nc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    uint32_t wadd = 0, btotal = 0;
    for (int i = 0; i < kThreads / 32; ++i) {
      if (i < w) wadd += s_warp[i];
      btotal += s_warp[i];
    }
    const uint32_t my_excl = x - (uint32_t)nc + wadd;
    // tile look-back (thread 0)
    if (t == 0) {
      const uint32_t excl = tile_lookback(lb, tile, btotal, err);
      s_excl = excl;
      if (tile == ntiles - 1) level_bounds[d + 2] = hi + (int)(excl + btotal);
    }
    __syncthreads();
    const long long child_base = (long long)hi + s_excl + my_excl;
    if (valid) {
      bool fits = child_base + nc <= node_cap;
      if (!fits) atomicOr(err, kErrNodes);
      int first = -1;
      if (internal && fits) {
        first = (int)child_base;
        int k = 0;
        const uint64_t pk = nkey[node];
        for (int v = 0; v < 8; ++v) {
          if (!(mask & (1u << v))) continue;
          int ci = first + k++;
          nkey[ci] = (pk << 3) | (uint64_t)v;
          nrange[ci] = make_int2(bnd[v], bnd[v + 1] - bnd[v]);
        }
      }
      wn[node].link = make_int4(first, (internal && fits) ? nc : 0, r.x, r.y);
      childbyte[node] = (uint8_t)((internal && fits) ? mask : 0u);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------
// Parallel build: every depth at once
// ---------------------------------------------------------------------------------------
// The same node set, order and records as k_tree_init + k_level, without a chain of levels.
// With the tree keys sorted, a depth-e cell is a contiguous run of bodies, and:
//   * the depth-e cell of body i holds more than L bodies exactly when some run of L + 1
//     consecutive bodies containing i shares its first e digits; the keys being sorted, a run
//     [j, j + L] shares as many digits as its end keys do. So with w(j) = digits shared by keys j
//     and j + L, E(i) = max of w(j) over j in [i - L, i] is the deepest such depth;
//   * a node of depth d >= 1 is a non-empty cell whose parent cell holds more than L bodies
//     (the parent's parent then does too), so a depth-d node starts at body i exactly when keys
//     i - 1 and i differ in the first d digits and d <= E(i) + 1 (and d <= 21): every depth
//     from (digits shared with key i - 1) + 1 to min(E(i) + 1, 21).
// The build counts node starts per depth for each tile of bodies (k_nodes_count), scans the
// counts of each depth over the tiles (k_nodes_scan), writes every node from the thread of its
// first body (k_nodes_write: index = level start + starts of its depth before it; its cell's
// end by a galloping search; its first child is node (d + 1, i); its parent is the last
// depth-(d - 1) node starting at or before i), and lets each parent's last child set the
// parent's child count and child byte (k_nodes_link).
constexpr int kPBThreads = 512;
constexpr int kPBWarps = kPBThreads / 32;
constexpr int kPBMaxLeaf = 64;  // halo of the window maxima; larger leaf capacities use k_level

// Octal digits (from the top) that two tree keys share; 21 when they are equal (the marker bit
// 63 is set in both).
__device__ __forceinline__ int common_digits(uint64_t a, uint64_t b) {
  const uint64_t x = a ^ b;
  return x ? (__clzll((long long)x) - 1) / 3 : kMaxDepth;
}

// Per-warp counts of node starts for each depth 1..21 (ballots only over the depths the warp's
// bodies start nodes at; a warp of 32 neighbouring bodies spans a few depths of the 21).
__device__ __forceinline__ void warp_start_counts(int lo, int hi, uint32_t (*s_wc)[kPBWarps]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wlo = __reduce_min_sync(0xffffffffu, lo), whi = __reduce_max_sync(0xffffffffu, hi);
  for (int d = 1 + lane; d <= kMaxDepth; d += 32)
    if (d < wlo || d > whi) s_wc[d - 1][w] = 0u;
  for (int d = wlo; d <= whi; ++d) {
    const unsigned b = __ballot_sync(0xffffffffu, lo <= d && d <= hi);
    if (lane == 0) s_wc[d - 1][w] = (uint32_t)__popc(b);
  }
}

// Start depths of the tile's bodies: lo | hi << 8 (none when lo > hi), and per-warp counts of
// starts for each depth 1..21 in s_wc.
__device__ void node_start_depths(const uint64_t* __restrict__ tkey, int n, int leaf_cap, int t0,
                                  uint32_t (*s_wc)[kPBWarps], uint32_t* span_out) {
  __shared__ uint64_t s_k[kPBThreads + 2 * kPBMaxLeaf];
  __shared__ int8_t s_w[kPBThreads + kPBMaxLeaf];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, L = leaf_cap;
  const int base = t0 - L;  // s_k[x - base] is key x, for x in [t0 - L, t0 + T + L)
  for (int x = t; x < kPBThreads + 2 * L; x += kPBThreads) {
    const int g = base + x;
    s_k[x] = (g >= 0 && g < n) ? tkey[g] : 0ull;
  }
  __syncthreads();
  for (int x = t; x < kPBThreads + L; x += kPBThreads) {  // w(j) for j in [t0 - L, t0 + T)
    const int j = base + x;
    s_w[x] = (int8_t)((j >= 0 && j + L < n) ? common_digits(s_k[x], s_k[x + L]) : -1);
  }
  __syncthreads();
  const int i = t0 + t;
  int lo = 1, hi = 0;
  if (i < n) {
    const uint64_t ki = s_k[i - base];
    const int lcp = i == 0 ? -1 : common_digits(s_k[i - 1 - base], ki);
    int e = -1;
    for (int q = 0; q <= L; ++q) e = max(e, (int)s_w[t + q]);  // j = i - L + q
    lo = max(lcp + 1, 1);
    hi = min(e + 1, kMaxDepth);
  }
  if (i < n) span_out[i] = (uint32_t)lo | ((uint32_t)hi << 8);
  warp_start_counts(lo, hi, s_wc);
  __syncthreads();
}

__global__ __launch_bounds__(kPBThreads) void k_nodes_count(const uint64_t* __restrict__ tkey, int n, int leaf_cap,
                                                            uint32_t* __restrict__ span,
                                                            uint32_t* __restrict__ tile_cnt, int ntiles) {
  __shared__ uint32_t s_wc[kMaxDepth][kPBWarps];
  node_start_depths(tkey, n, leaf_cap, blockIdx.x * kPBThreads, s_wc, span);
  if (threadIdx.x < kMaxDepth) {
    uint32_t c = 0;
    for (int q = 0; q < kPBWarps; ++q) c += s_wc[threadIdx.x][q];
    tile_cnt[(size_t)threadIdx.x * ntiles + blockIdx.x] = c;
  }
}

// Block d - 1 scans depth d's tile counts (exclusive, in place) and stores the depth's total.
__global__ __launch_bounds__(1024) void k_nodes_scan(uint32_t* __restrict__ tile_cnt, int ntiles,
                                                     uint32_t* __restrict__ totals) {
  __shared__ uint32_t s_warp[32];
  uint32_t* c = tile_cnt + (size_t)blockIdx.x * ntiles;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (ntiles + 1023) / 1024, a = min(ntiles, t * per), b = min(ntiles, a + per);
  uint32_t sum = 0;
  for (int q = a; q < b; ++q) sum += c[q];
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[w] = x;
  __syncthreads();
  if (w == 0) {
    const uint32_t v = s_warp[lane];
    uint32_t z = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += y;
    }
    s_warp[lane] = z - v;
    if (lane == 31) totals[blockIdx.x] = z;
  }
  __syncthreads();
  uint32_t run = x - sum + s_warp[w];
  for (int q = a; q < b; ++q) {
    const uint32_t v = c[q];
    c[q] = run;
    run += v;
  }
}

// Level starts (s_lb, from the depth totals) and, per depth and warp of this tile, the index of
// the warp's first node start (s_first); returns the node count.
__device__ long long node_first_indices(int n, uint32_t lo, uint32_t hi, const uint32_t* __restrict__ tile_excl,
                                        int ntiles, const uint32_t* __restrict__ totals, long long* s_lb,
                                        uint32_t (*s_first)[kPBWarps]) {
  const int t = threadIdx.x;
  if (t == 0) {
    s_lb[0] = 0;
    s_lb[1] = n > 0 ? 1 : 0;
    for (int d = 1; d <= kMaxDepth; ++d) s_lb[d + 1] = s_lb[d] + totals[d - 1];
  }
  warp_start_counts((int)lo, (int)hi, s_first);
  __syncthreads();
  if (t < kMaxDepth) {
    uint32_t run = (uint32_t)s_lb[t + 1] + tile_excl[(size_t)t * ntiles + blockIdx.x];
    for (int q = 0; q < kPBWarps; ++q) {
      const uint32_t v = s_first[t][q];
      s_first[t][q] = run;
      run += v;
    }
  }
  __syncthreads();
  return s_lb[kLevels];
}

// Node records from the thread of each node's first body: key, first body, parent, first
// child (node (d + 1, i); a node is internal exactly when d < the body's deepest start depth).
// The body counts, child counts and child bytes follow in k_nodes_link.
__global__ __launch_bounds__(kPBThreads) void k_nodes_write(const uint64_t* __restrict__ tkey, int n, int leaf_cap,
                                                            const uint32_t* __restrict__ span,
                                                            const uint32_t* __restrict__ tile_excl, int ntiles,
                                                            const uint32_t* __restrict__ totals,
                                                            uint64_t* __restrict__ nkey, int2* __restrict__ nrange,
                                                            WalkNode* __restrict__ wn, uint8_t* __restrict__ childbyte,
                                                            int* __restrict__ nparent, int* __restrict__ level_bounds,
                                                            long long node_cap, uint32_t* __restrict__ err) {
  __shared__ long long s_lb[kLevels + 1];
  __shared__ uint32_t s_first[kMaxDepth][kPBWarps];
  const int t = threadIdx.x, lane = t & 31;
  const int i = blockIdx.x * kPBThreads + t;
  const uint32_t sp = i < n ? span[i] : 1u;
  const int lo = (int)(sp & 0xFFu), hi = (int)(sp >> 8);
  const long long m = node_first_indices(n, (uint32_t)lo, (uint32_t)hi, tile_excl, ntiles, totals, s_lb, s_first);
  if (blockIdx.x == 0) {
    if (t <= kLevels + 1) level_bounds[t] = (int)min(s_lb[min(t, kLevels)], 0x7fffffffll);
    if (t == 0 && m > node_cap) atomicOr(err, kErrNodes);
  }
  if (m > node_cap) return;  // the host grows the arena and builds again
  const uint32_t lt = (1u << lane) - 1u;
  const uint64_t ki = i < n ? tkey[i] : 0ull;
  int child = -1;  // index of node (d + 1, i), when it exists
  // the warp's depths, and one above them for the parents of its shallowest nodes
  const int wlo = __reduce_min_sync(0xffffffffu, lo), whi = __reduce_max_sync(0xffffffffu, hi);
  for (int d = whi; d >= max(1, wlo - 1); --d) {
    const bool f = lo <= d && d <= hi;
    const unsigned b = __ballot_sync(0xffffffffu, f);
    const int idx = (int)s_first[d - 1][t >> 5] + __popc(b & lt);  // node (d, i) if f, else the next start
    if (child >= 0) nparent[child] = idx + (f ? 1 : 0) - 1;  // the last depth-d node starting at or before i
    if (f) {
      nkey[idx] = ki >> (3 * (kMaxDepth - d));
      nrange[idx] = make_int2(i, 0);
      wn[idx].link = make_int4(d < hi ? child : -1, 0, i, 0);
      childbyte[idx] = 0;
      child = idx;
    } else {
      child = -1;
    }
  }
  if (child >= 0) nparent[child] = 0;  // depth-1 nodes hang from the root
  if (i == 0) {
    const bool internal = n > leaf_cap;
    nkey[0] = 1ull;
    nrange[0] = make_int2(0, n);
    wn[0].link = make_int4(internal ? 1 : -1, 0, 0, n);
    childbyte[0] = 0;
    nparent[0] = -1;
  }
}

// Body counts, child counts and child bytes, one thread per node. Siblings are contiguous and
// their cells adjacent, so a node's cell ends where its next sibling's starts, and a last
// child's where its parent's ends (the climb passes only through last children: about 1.3
// nodes on average). The last child of each parent (the next node has another parent) also
// counts its siblings from the parent's first child and ORs their digits. The upsweep's arrival
// counters are zeroed here as well (the parent links it needs are k_nodes_write's), so the
// all-depths build needs no separate k_upsweep_links.
__global__ __launch_bounds__(kThreads) void k_nodes_link(const int* __restrict__ level_bounds,
                                                         const uint64_t* __restrict__ nkey,
                                                         const int* __restrict__ nparent, int2* __restrict__ nrange,
                                                         WalkNode* __restrict__ wn, uint8_t* __restrict__ childbyte,
                                                         uint32_t* __restrict__ arrived,
                                                         const uint32_t* __restrict__ err) {
  if (*err & kErrNodes) return;
  const int m = level_bounds[kLevels];
  const int n = nrange[0].y;
  if (blockIdx.x == 0 && threadIdx.x == 0) arrived[0] = 0u;
  auto last_child = [&](int j) { return j + 1 >= m || nparent[j + 1] != nparent[j]; };
  for (int j = 1 + blockIdx.x * kThreads + threadIdx.x; j < m; j += gridDim.x * kThreads) {
    arrived[j] = 0u;
    const bool last = last_child(j);
    int a = j;
    bool up = last;
    while (up) {
      a = nparent[a];
      if (a == 0) break;
      up = last_child(a);
    }
    const int first = nrange[j].x;
    const int cnt = (up ? n : nrange[a + 1].x) - first;  // up: the climb reached the root
    nrange[j].y = cnt;
    wn[j].link.w = cnt;
    if (!last) continue;
    const int p = nparent[j];
    const int fc = wn[p].link.x;
    uint32_t mask = 0;
    for (int c = fc; c <= j; ++c) mask |= 1u << (uint32_t)(nkey[c] & 7ull);
    wn[p].link.y = j - fc + 1;
    childbyte[p] = (uint8_t)mask;
  }
}

// ---------------------------------------------------------------------------------------
// upsweep
// ---------------------------------------------------------------------------------------

// Parallel-axis quadrupole contribution of one child (or member body) of mass m at offset x
// from the node's centre of mass, the reference's formulas (src/HashedOctree.cpp:778-808).
__device__ __forceinline__ void quad_add(float q[6], float m, float x, float y, float z) {
  const float m3 = 3.f * m;
  q[1] = fmaf(m3 * x, y, q[1]);
  q[2] = fmaf(m3 * x, z, q[2]);
  q[4] = fmaf(m3 * y, z, q[4]);
  const float r2m = m * fmaf(x, x, fmaf(y, y, z * z));
  q[0] += fmaf(m3 * x, x, -r2m);
  q[3] += fmaf(m3 * y, y, -r2m);
  q[5] += fmaf(m3 * z, z, -r2m);
}

// A child's upsweep record as written by another thread of the same launch: read through L2
// (an L1 line could hold a stale copy fetched for a neighbouring node).
__device__ __forceinline__ NodeUp load_nodeup(const NodeUp* p) {
  const float4* f = reinterpret_cast<const float4*>(p);
  const float4 a = __ldcg(f), b = __ldcg(f + 1), c = __ldcg(f + 2), d = __ldcg(f + 3);
  NodeUp u;
  u.com_hi[0] = a.x;
  u.com_hi[1] = a.y;
  u.com_hi[2] = a.z;
  u.mass_hi = a.w;
  u.com_lo[0] = b.x;
  u.com_lo[1] = b.y;
  u.com_lo[2] = b.z;
  u.mass_lo = b.w;
  u.q[0] = c.x;
  u.q[1] = c.y;
  u.q[2] = c.z;
  u.q[3] = c.w;
  u.q[4] = d.x;
  u.q[5] = d.y;
  u.min_rank = __float_as_uint(d.z);
  u.pad = __float_as_uint(d.w);
  return u;
}

// The multipole of one node at depth d (computeTreeBaryCenters / computeNodeBaryCenters,
// src/HashedOctree.cpp:721-855, as intended; or the literal pseudo-barycentres). A leaf
// combines its member bodies, an internal node its children, whose records are complete.
// kPrefetch (small trees, where the climb's latency is the upsweep's time): an internal node
// loads all its children's records at once before combining them, one L2 round trip instead of
// one per child and pass; the arithmetic and its order are the same, so are the results.
template <bool kPrefetch>
__device__ void upsweep_node(int node, int d, int mode, const float4* __restrict__ tpos,
                             const uint32_t* __restrict__ tslot, WalkNode* __restrict__ wn, NodeUp* __restrict__ nf,
                             const Geom* __restrict__ g, const uint16_t* __restrict__ body_sys) {
  {
    const int4 link = wn[node].link;
    // batched ensembles: the node's system (that of its first body) sets the root edge
    const double edge = ldexp(body_sys ? g[body_sys[link.z]].tedge : g->tedge, -d);
    const float s2 = (float)(edge * edge);
    FF mass = {0.f, 0.f}, com[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    float q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    uint32_t min_rank = 0xffffffffu;
    bool single = false;
    if (link.y == 0) {  // leaf: members are tree-order bodies [link.z, link.z + link.w)
      if (mode == BH_MULTIPOLE_LITERAL) {
        int first = link.z;
        for (int b = link.z; b < link.z + link.w; ++b) {
          mass = ff_add(mass, {tpos[b].w, 0.f});
          const uint32_t rk = tslot[b];
          if (rk < min_rank) {
            min_rank = rk;
            first = b;
          }
        }
        const float4 p = tpos[first];
        com[0] = {p.x, 0.f};
        com[1] = {p.y, 0.f};
        com[2] = {p.z, 0.f};
        single = link.w == 1;
      } else if (link.w == 1) {
        const float4 p = tpos[link.z];
        com[0] = {p.x, 0.f};
        com[1] = {p.y, 0.f};
        com[2] = {p.z, 0.f};
        mass = {p.w, 0.f};
        min_rank = tslot[link.z];
        single = true;
      } else {
        // members in batches of four: the batch's loads are issued together before the
        // dependent float-float sums (same summation order as one member at a time)
        const int end = link.z + link.w;
        for (int b0 = link.z; b0 < end; b0 += 4) {
          float4 pb[4];
          uint32_t rb[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            pb[j] = b0 + j < end ? tpos[b0 + j] : make_float4(0.f, 0.f, 0.f, 0.f);
            rb[j] = b0 + j < end ? tslot[b0 + j] : 0xffffffffu;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (b0 + j >= end) break;
            const float4 p = pb[j];
            mass = ff_add(mass, {p.w, 0.f});
            com[0] = ff_add(com[0], ff_prod(p.x, p.w));
            com[1] = ff_add(com[1], ff_prod(p.y, p.w));
            com[2] = ff_add(com[2], ff_prod(p.z, p.w));
            min_rank = min(min_rank, rb[j]);
          }
        }
        if (mass.hi != 0.f)
          for (int a = 0; a < 3; ++a) com[a] = ff_div(com[a], mass);
        for (int b0 = link.z; b0 < end; b0 += 4) {
          float4 pb[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) pb[j] = b0 + j < end ? tpos[b0 + j] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (b0 + j >= end) break;
            const float4 p = pb[j];
            quad_add(q, p.w, (p.x - com[0].hi) - com[0].lo, (p.y - com[1].hi) - com[1].lo,
                     (p.z - com[2].hi) - com[2].lo);
          }
        }
      }
    } else if (kPrefetch) {
      NodeUp ch[8];
      int cw[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (k < link.y) {
          ch[k] = load_nodeup(nf + link.x + k);
          cw[k] = mode == BH_MULTIPOLE_LITERAL ? 0 : wn[link.x + k].link.w;
        }
      if (mode == BH_MULTIPOLE_LITERAL) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (k < link.y) {
            mass = ff_add(mass, {ch[k].mass_hi, ch[k].mass_lo});
            if (ch[k].min_rank < min_rank) {
              min_rank = ch[k].min_rank;
              for (int a = 0; a < 3; ++a) com[a] = {ch[k].com_hi[a], ch[k].com_lo[a]};
            }
          }
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (k < link.y) {
            const FF m = {ch[k].mass_hi, ch[k].mass_lo};
            mass = ff_add(mass, m);
            for (int a = 0; a < 3; ++a) com[a] = ff_add(com[a], ff_mul({ch[k].com_hi[a], ch[k].com_lo[a]}, m));
            min_rank = min(min_rank, ch[k].min_rank);
          }
        if (mass.hi != 0.f)
          for (int a = 0; a < 3; ++a) com[a] = ff_div(com[a], mass);
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (k < link.y) {
            quad_add(q, ch[k].mass_hi, (ch[k].com_hi[0] - com[0].hi) + (ch[k].com_lo[0] - com[0].lo),
                     (ch[k].com_hi[1] - com[1].hi) + (ch[k].com_lo[1] - com[1].lo),
                     (ch[k].com_hi[2] - com[2].hi) + (ch[k].com_lo[2] - com[2].lo));
            if (cw[k] > 1)
              for (int j = 0; j < 6; ++j) q[j] += ch[k].q[j];
          }
      }
    } else {
      if (mode == BH_MULTIPOLE_LITERAL) {
        for (int c = link.x; c < link.x + link.y; ++c) {
          const NodeUp ch = load_nodeup(nf + c);
          mass = ff_add(mass, {ch.mass_hi, ch.mass_lo});
          if (ch.min_rank < min_rank) {
            min_rank = ch.min_rank;
            for (int a = 0; a < 3; ++a) com[a] = {ch.com_hi[a], ch.com_lo[a]};
          }
        }
      } else {
        // (batching the children's loads like the leaf members' measured slower here)
        for (int c = link.x; c < link.x + link.y; ++c) {
          const NodeUp ch = load_nodeup(nf + c);
          const FF m = {ch.mass_hi, ch.mass_lo};
          mass = ff_add(mass, m);
          for (int a = 0; a < 3; ++a) com[a] = ff_add(com[a], ff_mul({ch.com_hi[a], ch.com_lo[a]}, m));
          min_rank = min(min_rank, ch.min_rank);
        }
        if (mass.hi != 0.f)
          for (int a = 0; a < 3; ++a) com[a] = ff_div(com[a], mass);
        for (int c = link.x; c < link.x + link.y; ++c) {
          const NodeUp ch = load_nodeup(nf + c);
          quad_add(q, ch.mass_hi, (ch.com_hi[0] - com[0].hi) + (ch.com_lo[0] - com[0].lo),
                   (ch.com_hi[1] - com[1].hi) + (ch.com_lo[1] - com[1].lo),
                   (ch.com_hi[2] - com[2].hi) + (ch.com_lo[2] - com[2].lo));
          if (wn[c].link.w > 1)
            for (int k = 0; k < 6; ++k) q[k] += ch.q[k];
        }
      }
    }
    NodeUp out;
    for (int a = 0; a < 3; ++a) {
      out.com_hi[a] = com[a].hi;
      out.com_lo[a] = com[a].lo;
    }
    out.mass_hi = mass.hi;
    out.mass_lo = mass.lo;
    for (int k = 0; k < 6; ++k) out.q[k] = q[k];
    out.min_rank = min_rank;
    out.pad = 0;
    nf[node] = out;
    wn[node].mac = make_float4(com[0].hi, com[1].hi, com[2].hi, single ? -s2 : s2);
    wn[node].mq = make_float4(mass.hi, q[0], q[1], q[2]);
    wn[node].q2 = make_float4(q[3], q[4], q[5], 0.f);
  }
}

// Parent links of the tree just built, and the arrival counters of the upsweep.
__global__ __launch_bounds__(kThreads) void k_upsweep_links(const int* __restrict__ level_bounds,
                                                            const WalkNode* __restrict__ wn, int* __restrict__ parent,
                                                            uint32_t* __restrict__ arrived,
                                                            const uint32_t* __restrict__ err) {
  if (*err & kErrNodes) return;
  const int m = level_bounds[kLevels], roots = level_bounds[1];
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < m; i += gridDim.x * kThreads) {
    arrived[i] = 0u;
    if (i < roots) parent[i] = -1;
    const int4 link = wn[i].link;
    for (int c = link.x; c < link.x + link.y; ++c) parent[c] = i;
  }
}

// The bottom-up multipole pass in one launch. A thread per leaf computes the leaf, then climbs:
// having published a node, it counts itself in at the parent; the thread
// that completes the parent's count (the last of the children to finish) computes the parent
// from all its children, in child order, and goes on up. Every node is computed once, from
// complete children, with the arithmetic and order of a level-by-level pass, and no thread
// ever waits for another.
template <bool kPrefetch>
__global__ __launch_bounds__(kThreads) void k_upsweep(int mode, const int* __restrict__ level_bounds,
                                                      const uint64_t* __restrict__ nkey,
                                                      const int* __restrict__ parent, uint32_t* __restrict__ arrived,
                                                      const float4* __restrict__ tpos,
                                                      const uint32_t* __restrict__ tslot,
                                                      WalkNode* __restrict__ wn, NodeUp* __restrict__ nf,
                                                      const Geom* __restrict__ g, const uint16_t* __restrict__ body_sys,
                                                      const uint32_t* __restrict__ err, Counters* __restrict__ ctr) {
  if (*err & kErrNodes) return;
  const int m = level_bounds[kLevels];
  unsigned deepest = 0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < m; i += gridDim.x * kThreads) {
    if (wn[i].link.y != 0) continue;  // internal: computed by its last child's thread
    int node = i;
    int d = (63 - __clzll((long long)nkey[i])) / 3;
    deepest = max(deepest, (unsigned)d);
    for (;;) {
      upsweep_node<kPrefetch>(node, d, mode, tpos, tslot, wn, nf, g, body_sys);
      const int p = parent[node];
      if (p < 0) break;
      // the parent's child count (written by the build) can be read before the arrival atomic
      const int pchildren = kPrefetch ? wn[p].link.y : 0;
      // acquire-release: this node's stores are visible to the thread that completes the
      // parent, and that thread sees every child's stores
      unsigned prev;
      asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(prev) : "l"(arrived + p) : "memory");
      if (prev + 1u < (unsigned)(kPrefetch ? pchildren : wn[p].link.y)) break;
      node = p;
      --d;
    }
  }
  deepest = __reduce_max_sync(0xffffffffu, deepest);
  if ((threadIdx.x & 31) == 0 && deepest > 0) atomicMax(&ctr->max_depth, deepest);
}

// ---------------------------------------------------------------------------------------
// node hash table (replaces the std::unordered_map of LinearHashedOctree,
// src/HashedOctree.hpp:134; lookups as in lookUpNode, src/HashedOctree.cpp:111-115)
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ size_t hash_slot(uint64_t key, size_t mask) {
  return (size_t)((key * 0x9E3779B97F4A7C15ull) >> 17) & mask;
}

constexpr int kHashProbeLimit = 4096;

__global__ __launch_bounds__(kThreads) void k_hash_insert(const uint64_t* __restrict__ nkey,
                                                          const int* __restrict__ level_bounds,
                                                          unsigned long long* __restrict__ hk,
                                                          int* __restrict__ hv, size_t cap,
                                                          long long node_cap, uint32_t* __restrict__ err) {
  const int m = (int)min((long long)level_bounds[kLevels], node_cap);
  const size_t mask = cap - 1;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < m; i += gridDim.x * kThreads) {
    unsigned long long key = nkey[i];
    size_t h = hash_slot(key, mask);
    int probe = 0;
    for (;;) {
      unsigned long long prev = atomicCAS(&hk[h], 0ull, key);
      if (prev == 0ull || prev == key) {
        hv[h] = i;
        break;
      }
      if (++probe >= kHashProbeLimit) {
        atomicOr(err, kErrHash);
        break;
      }
      h = (h + 1) & mask;
    }
  }
}

__global__ void k_hash_lookup(const unsigned long long* __restrict__ hk, const int* __restrict__ hv, size_t cap,
                              uint64_t key, int* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const size_t mask = cap - 1;
  size_t h = hash_slot(key, mask);
  int res = -1;
  for (int probe = 0; probe < kHashProbeLimit; ++probe) {
    unsigned long long k = hk[h];
    if (k == key) {
      res = hv[h];
      break;
    }
    if (k == 0ull) break;
    h = (h + 1) & mask;
  }
  *out = res;
}

// Register-only FMA loop for the measured FP32 roofline (8 independent chains per thread).
__global__ __launch_bounds__(kThreads) void k_fp32_peak(float* sink, int iters) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fmaf(a0, b, c);
      a1 = fmaf(a1, b, c);
      a2 = fmaf(a2, b, c);
      a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c);
      a5 = fmaf(a5, b, c);
      a6 = fmaf(a6, b, c);
      a7 = fmaf(a7, b, c);
    }
  }
  float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 12345.678f) sink[0] = r;  // keeps the loop alive; never true for these inputs
}

// ---------------------------------------------------------------------------------------
// batched ensembles: system s owns the fixed body range [off[s], off[s + 1])
// ---------------------------------------------------------------------------------------

// OctantBounds of every system, one block per system: FP64 sums in a fixed order (thread
// stride, then a fixed tree), FP32 maxima of |p|, then the same centre / size / geometry
// formulas as k_bounds_final.
__global__ __launch_bounds__(kThreads) void k_batch_bounds(const float4* __restrict__ pos,
                                                           const uint32_t* __restrict__ off, double edge_factor,
                                                           Geom* __restrict__ sys_geom) {
  const int s = blockIdx.x;
  const int b0 = (int)off[s], b1 = (int)off[s + 1];
  double sx = 0, sy = 0, sz = 0;
  float mx = 0.f, my = 0.f, mz = 0.f;
  for (int i = b0 + threadIdx.x; i < b1; i += kThreads) {
    const float4 p = pos[i];
    sx = __dadd_rn(sx, (double)p.x);
    sy = __dadd_rn(sy, (double)p.y);
    sz = __dadd_rn(sz, (double)p.z);
    mx = fmaxf(mx, fabsf(p.x));
    my = fmaxf(my, fabsf(p.y));
    mz = fmaxf(mz, fabsf(p.z));
  }
  __shared__ double sh[6][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sx = __dadd_rn(sx, __shfl_down_sync(0xffffffffu, sx, o));
    sy = __dadd_rn(sy, __shfl_down_sync(0xffffffffu, sy, o));
    sz = __dadd_rn(sz, __shfl_down_sync(0xffffffffu, sz, o));
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    my = fmaxf(my, __shfl_down_sync(0xffffffffu, my, o));
    mz = fmaxf(mz, __shfl_down_sync(0xffffffffu, mz, o));
  }
  if (lane == 0) {
    sh[0][w] = sx;
    sh[1][w] = sy;
    sh[2][w] = sz;
    sh[3][w] = mx;
    sh[4][w] = my;
    sh[5][w] = mz;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double c[3], m[3];
  for (int a = 0; a < 3; ++a) {
    c[a] = sh[a][0];
    m[a] = sh[3 + a][0];
    for (int k = 1; k < kThreads / 32; ++k) {
      c[a] = __dadd_rn(c[a], sh[a][k]);
      m[a] = fmax(m[a], sh[3 + a][k]);
    }
  }
  const double nn = (double)(b1 - b0);
  if (nn != 0) {
    const double inv = __ddiv_rn(1.0, nn);
    for (int a = 0; a < 3; ++a) c[a] = __dmul_rn(c[a], inv);
  }
  double S = 0;
  for (int a = 0; a < 3; ++a) {
    const double v = __dsub_rn(m[a], c[a]);
    if (v > S) S = v;
  }
  Geom& g = sys_geom[s];
  for (int a = 0; a < 3; ++a) g.center[a] = c[a];
  g.size = S;
  g.frac = __ddiv_rn(2097152.0, __dmul_rn(2.0, S));
  fill_tree_geom(g, c, __dmul_rn(S, edge_factor));
}

// Secondary sort key: the system of the body each sorted element came from. A stable sort of
// the key-sorted elements by it groups them back into their systems, in key order.
__global__ __launch_bounds__(kThreads) void k_sys_keys(const uint32_t* __restrict__ vals, int n,
                                                       const uint16_t* __restrict__ body_sys,
                                                       uint64_t* __restrict__ k2) {
  const int j = blockIdx.x * kThreads + threadIdx.x;
  if (j < n) k2[j] = (uint64_t)body_sys[vals[j]];
}

// Tree-order positions and tree keys of a batched ensemble: the (system, key) sort leaves the
// permutation in tslot, the keys themselves are gathered from their per-slot copy.
__global__ __launch_bounds__(kThreads) void k_gather_tree_keys(const uint32_t* __restrict__ tslot, int n,
                                                               const float4* __restrict__ pos,
                                                               const uint64_t* __restrict__ key_by_slot,
                                                               float4* __restrict__ tpos,
                                                               uint64_t* __restrict__ tkey) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = tslot[i];
  tpos[i] = pos[s];
  tkey[i] = key_by_slot[s];
}

// One root per system at depth 0, in system order.
__global__ void k_tree_init_batch(int nsys, const uint32_t* __restrict__ off, uint64_t* __restrict__ nkey,
                                  int2* __restrict__ nrange, int* __restrict__ level_bounds,
                                  uint32_t* __restrict__ level_tile_ctr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nsys) {
    nkey[t] = 1ull;
    nrange[t] = make_int2((int)off[t], (int)(off[t + 1] - off[t]));
  }
  if (t < kLevels) level_tile_ctr[t] = 0;
  if (t <= kLevels + 1) level_bounds[t] = (t == 0) ? 0 : (t == 1 ? nsys : -1);
}

inline int grid_for(long long n) { return (int)((n + kThreads - 1) / kThreads); }

}  // namespace

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------

void launch_bounds(bh_ctx* c, const float4* pos, int n, double edge_factor) {
  c->launches += 2;
  k_bounds_partial<<<c->bounds_blocks, kThreads, 0, c->stream>>>(pos, n, c->bounds_partial);
  k_bounds_final<<<1, 32, 0, c->stream>>>(c->bounds_partial, c->bounds_blocks, n, edge_factor, c->geom);
}

void launch_set_geom(bh_ctx* c, const double center[3], double size, const double tcenter[3], double tedge) {
  c->launches += 1;
  k_set_geom<<<1, 32, 0, c->stream>>>(c->geom, center[0], center[1], center[2], size, tcenter[0], tcenter[1],
                                      tcenter[2], tedge);
}

void launch_morton(bh_ctx* c, const float4* pos, int n, uint64_t* keys, uint32_t* idx, bool batch) {
  if (n > 0) c->launches += 1;
  if (n > 0)
    k_morton<<<grid_for(n), kThreads, 0, c->stream>>>(pos, n, batch ? c->sys_geom : c->geom,
                                                       batch ? c->body_sys : nullptr, keys, idx);
}

void launch_decode_morton(bh_ctx* c, const uint64_t* keys, int n, double size, double* pos3) {
  if (n <= 0) return;
  c->launches += 1;
  k_decode_morton<<<grid_for(n), kThreads, 0, c->stream>>>(keys, n, size, pos3);
}

void launch_treekey(bh_ctx* c, const float4* pos, int n, uint64_t* tkeys, uint32_t* tidx) {
  if (n > 0) c->launches += 1;
  if (n > 0) k_treekey<<<grid_for(n), kThreads, 0, c->stream>>>(pos, n, c->geom, tkeys, tidx);
}

void launch_gather(bh_ctx* c, const uint32_t* perm, int n, const float4* pin, const float4* vin, float4* pout,
                   float4* vout) {
  if (n > 0) c->launches += 1;
  if (n > 0) k_gather<<<grid_for(n), kThreads, 0, c->stream>>>(perm, n, pin, vin, pout, vout);
}

void launch_gather_kd_treekey(bh_ctx* c, const uint32_t* perm, int n, const float4* pin, const float4* vin,
                              const float4* acc, int acc_follows_body, float dt, float4* pout, float4* vout,
                              uint64_t* tkeys, uint32_t* tidx, bool batch) {
  if (n > 0) c->launches += 1;
  if (n > 0)
    k_gather_kd_treekey<<<grid_for(n), kThreads, 0, c->stream>>>(
        perm, n, pin, vin, acc, acc_follows_body, dt, 0.5f * dt, batch ? c->sys_geom : c->geom,
        batch ? c->body_sys : nullptr, pout, vout, tkeys, tidx);
}

void launch_kick_drift(bh_ctx* c, float4* pos, float4* vel, const float4* acc, int n, float dt, int drift) {
  if (n > 0) c->launches += 1;
  if (n > 0) k_kick_drift<<<grid_for(n), kThreads, 0, c->stream>>>(pos, vel, acc, n, dt, 0.5f * dt, drift);
}

void launch_gather_tree(bh_ctx* c, const uint32_t* tslot, int n, const float4* pos, float4* tpos) {
  if (n > 0) c->launches += 1;
  if (n > 0) k_gather_tree<<<grid_for(n), kThreads, 0, c->stream>>>(tslot, n, pos, tpos);
}

// Function attributes set once per process, before any stream capture (none at present).
void tree_init() {}

// Single trees with leaves of at most kPBMaxLeaf bodies: every depth at once (k_nodes_*), parent
// links and the upsweep's counters included; otherwise the level build.
bool builds_all_depths(int n, int leaf_cap, bool batch) { return !batch && n >= 1 && leaf_cap <= kPBMaxLeaf; }

void launch_build(bh_ctx* c, int n, int leaf_cap, bool batch) {
  if (builds_all_depths(n, leaf_cap, batch)) {
    // every depth at once: counts per tile and depth (in lb_level), their scans (totals in
    // level_tile_ctr), the node records (start depths of each body in vals[1], free after the
    // sorts), then child counts and bytes
    const int ntiles = (n + kPBThreads - 1) / kPBThreads;
    uint32_t* span = c->vals[1];
    uint32_t* tile = c->lb_level;
    uint32_t* totals = c->level_tile_ctr;
    c->launches += 4;
    k_nodes_count<<<ntiles, kPBThreads, 0, c->stream>>>(c->tkey, n, leaf_cap, span, tile, ntiles);
    k_nodes_scan<<<kMaxDepth, 1024, 0, c->stream>>>(tile, ntiles, totals);
    k_nodes_write<<<ntiles, kPBThreads, 0, c->stream>>>(c->tkey, n, leaf_cap, span, tile, ntiles, totals, c->nkey,
                                                        c->nrange, c->wnode, c->nchildbyte, c->nparent,
                                                        c->level_bounds, (long long)c->node_cap, c->err);
    const int lgrid = (int)std::min<size_t>((size_t)c->sms * 8, (c->node_cap + kThreads - 1) / kThreads);
    k_nodes_link<<<lgrid, kThreads, 0, c->stream>>>(c->level_bounds, c->nkey, c->nparent, c->nrange, c->wnode,
                                                    c->nchildbyte, c->narrived, c->err);
    return;
  }
  c->launches += 1 + kLevels;
  if (batch)
    k_tree_init_batch<<<(max(c->nsys, kLevels + 2) + 255) / 256, 256, 0, c->stream>>>(
        c->nsys, c->sys_off, c->nkey, c->nrange, c->level_bounds, c->level_tile_ctr);
  else
    k_tree_init<<<1, 64, 0, c->stream>>>(n, c->nkey, c->nrange, c->level_bounds, c->level_tile_ctr);
  const int max_tiles = c->lb_level_tiles;
  cudaMemsetAsync(c->lb_level, 0, sizeof(uint32_t) * (size_t)kLevels * max_tiles, c->stream);
  const int grid = c->sms * 4;
  for (int d = 0; d < kLevels; ++d)
    k_level<<<grid, kThreads, 0, c->stream>>>(d, c->tkey, leaf_cap, c->nkey, c->nrange, c->wnode, c->nchildbyte,
                                              c->level_bounds, c->level_tile_ctr,
                                              c->lb_level + (size_t)d * max_tiles, (long long)c->node_cap, c->err);
}

#ifndef BH_UPSWEEP_PREFETCH_MAX
#define BH_UPSWEEP_PREFETCH_MAX 65536
#endif
// systems of at most this many bodies climb with the children's records prefetched
constexpr int kUpsweepPrefetchMaxBodies = BH_UPSWEEP_PREFETCH_MAX;

void launch_upsweep(bh_ctx* c, int n, int leaf_cap, int mode, bool batch) {
  if (n <= 0) return;
  // a thread for every two bodies, about one per node or more at leaf capacity >= 2 (the climbs
  // want a thread per leaf: at N = 2^22 a fixed 8 blocks per SM took 0.39 ms, this 0.27 ms, the
  // level-by-level pass it replaces 0.29 ms; at N = 2^25 a fixed 32 blocks per SM took 2.65 ms,
  // this 1.54 ms)
  const int grid = std::max(c->sms * 8, (n / 2 + kThreads - 1) / kThreads);
  // parent links and zeroed arrival counters: written by the all-depths build itself, or here
  // after the level build
  if (!builds_all_depths(n, leaf_cap, batch)) {
    c->launches += 1;
    k_upsweep_links<<<grid, kThreads, 0, c->stream>>>(c->level_bounds, c->wnode, c->nparent, c->narrived, c->err);
  }
  c->launches += 1;
  // the prefetching climb holds eight children's records in registers (one block per SM): two
  // threads per body there (about one per node at leaf capacity 1), at least a block per SM
  const bool prefetch = n <= kUpsweepPrefetchMaxBodies;
  auto upsweep = prefetch ? k_upsweep<true> : k_upsweep<false>;
  const int ugrid = prefetch ? std::max(c->sms, (2 * n + kThreads - 1) / kThreads) : grid;
  upsweep<<<ugrid, kThreads, 0, c->stream>>>(mode, c->level_bounds, c->nkey, c->nparent, c->narrived, c->tpos,
                                              c->tslot, c->wnode, c->nup, batch ? c->sys_geom : c->geom,
                                              batch ? c->body_sys : nullptr, c->err, c->counters);
}

void launch_batch_bounds(bh_ctx* c, const float4* pos, double edge_factor) {
  c->launches += 1;
  k_batch_bounds<<<c->nsys, kThreads, 0, c->stream>>>(pos, c->sys_off, edge_factor, c->sys_geom);
}

void launch_gather_tree_keys(bh_ctx* c, const uint32_t* tslot, int n, const float4* pos,
                             const uint64_t* key_by_slot, float4* tpos, uint64_t* tkey) {
  if (n <= 0) return;
  c->launches += 1;
  k_gather_tree_keys<<<grid_for(n), kThreads, 0, c->stream>>>(tslot, n, pos, key_by_slot, tpos, tkey);
}

void launch_sys_keys(bh_ctx* c, const uint32_t* vals, int n, uint64_t* k2) {
  if (n <= 0) return;
  c->launches += 1;
  k_sys_keys<<<grid_for(n), kThreads, 0, c->stream>>>(vals, n, c->body_sys, k2);
}

void launch_hash(bh_ctx* c) {
  cudaMemsetAsync(c->hash_keys, 0, sizeof(uint64_t) * c->hash_cap, c->stream);
  c->launches += 1;
  k_hash_insert<<<c->sms * 8, kThreads, 0, c->stream>>>(c->nkey, c->level_bounds, (unsigned long long*)c->hash_keys,
                                                     c->hash_vals, c->hash_cap, (long long)c->node_cap, c->err);
}

void launch_lookup(bh_ctx* c, uint64_t key, int* out_index) {
  c->launches += 1;
  k_hash_lookup<<<1, 32, 0, c->stream>>>((const unsigned long long*)c->hash_keys, c->hash_vals, c->hash_cap, key,
                                         out_index);
}

void launch_fp32_peak(cudaStream_t st, float* sink, int blocks) {
  k_fp32_peak<<<blocks, kThreads, 0, st>>>(sink, 4096);
}

}  // namespace bh
