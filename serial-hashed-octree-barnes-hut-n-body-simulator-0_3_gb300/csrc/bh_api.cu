// The C ABI of include/bhgpu.h: context, state transfer, the per-stage entry points that
// mirror the reference's calls, and the fused per-step driver.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "bh_internal.cuh"

using bh::kLevels;

// Host helpers shared with the other translation units (declared in bh_internal.cuh).
namespace bh {

bh_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return BH_OK;
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? BH_ERR_OOM : BH_ERR_DEVICE;
}

bh_status last_launch() { return cuda_status(cudaGetLastError()); }

bh_status err_to_status(uint32_t e) {
  for (int bit = 0; bit < 8; ++bit)
    if (e & (1u << bit)) return (bh_status)(bit + 3);
  return BH_OK;
}

__global__ void k_iota(uint32_t* v, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

bh_status ensure_nodes(bh_ctx* c, size_t need) {
  if (c->node_cap >= need && c->nkey) return BH_OK;
  for (int k = 0; k < 2; ++k)  // captured graphs hold the old node pointers
    for (cudaGraphExec_t* g : {&c->graph[k], &c->host_graph[k]})
      if (*g) {
        cudaGraphExecDestroy(*g);
        *g = nullptr;
      }
  size_t cap = std::max<size_t>(need, 1024);
  dfree(c->nkey);
  dfree(c->nrange);
  dfree(c->wnode);
  dfree(c->nup);
  dfree(c->nchildbyte);
  dfree(c->nparent);
  dfree(c->narrived);
  dfree(c->hash_keys);
  dfree(c->hash_vals);
  c->hash_cap = 0;
  c->hash_valid = false;
  c->node_cap = 0;
  BH_TRY(dalloc(&c->nkey, cap));
  BH_TRY(dalloc(&c->nrange, cap));
  BH_TRY(dalloc(&c->wnode, cap));
  BH_TRY(dalloc(&c->nup, cap));
  BH_TRY(dalloc(&c->nchildbyte, cap));
  BH_TRY(dalloc(&c->nparent, cap));
  BH_TRY(dalloc(&c->narrived, cap));
  c->node_cap = cap;
  c->tree_valid = false;
  return BH_OK;
}

bh_status ensure_hash(bh_ctx* c) {
  size_t want = 1024;
  while (want < 2 * c->node_cap) want <<= 1;
  if (c->hash_cap >= want && c->hash_keys) return BH_OK;
  dfree(c->hash_keys);
  dfree(c->hash_vals);
  c->hash_cap = 0;
  BH_TRY(dalloc(&c->hash_keys, want));
  BH_TRY(dalloc(&c->hash_vals, want));
  c->hash_cap = want;
  return BH_OK;
}

// Reads the device error word (and the counters) after finishing the stream.
bh_status sync_and_check(bh_ctx* c, uint32_t* err_out) {
  cudaMemcpyAsync(c->h_err, c->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(c->h_counters, c->counters, sizeof(bh::Counters), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(c->h_level_bounds, c->level_bounds, sizeof(int) * (kLevels + 2), cudaMemcpyDeviceToHost,
                  c->stream);
  BH_TRY(cuda_status(cudaStreamSynchronize(c->stream)));
  if (err_out) *err_out = *c->h_err;
  return BH_OK;
}

void clear_device_flags(bh_ctx* c) {
  cudaMemsetAsync(c->err, 0, sizeof(uint32_t), c->stream);
  cudaMemsetAsync(c->counters, 0, sizeof(bh::Counters), c->stream);
}

size_t initial_node_cap(size_t n) { return std::max<size_t>(2 * n + 64, 1024); }

// Tree over the current bodies (slot order pos) with the tree geometry already in c->geom:
// tree keys -> sort -> tree-order positions -> node discovery -> multipole pass.
void enqueue_tree(bh_ctx* c, const float4* pos, int n, int leaf_cap, int mode, bool keys_ready) {
  if (!keys_ready) bh::launch_treekey(c, pos, n, c->tkey, c->tslot);
  uint64_t* ko;
  uint32_t* vo;
  bh::radix_sort_pairs(c, c->tkey, c->tslot, c->keys[1], c->vals[1], n, c->stream, &ko, &vo);
  bh::launch_gather_tree(c, c->tslot, n, pos, c->tpos);
}

void record(bh_ctx* c, bh_stats* st, int k) {
  if (st) cudaEventRecord(c->stage_ev[k], c->stream);
}

float elapsed(bh_ctx* c, int a, int b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, c->stage_ev[a], c->stage_ev[b]) != cudaSuccess) {
    cudaGetLastError();  // a timing that cannot be read is reported as 0, not as a launch error
    ms = 0.f;
  }
  return ms;
}

}  // namespace bh

using namespace bh;

namespace {
constexpr size_t kMaxBodies = (1u << 30) - 1;  // sort look-back words hold 30-bit counts
void destroy_graphs(bh_ctx* c);
bool same_params(const bh_params& a, const bh_params& b);
}  // namespace

extern "C" {

const char* bh_status_string(bh_status s) {
  switch (s) {
    case BH_OK: return "ok";
    case BH_ERR_INVALID_ARG: return "invalid argument";
    case BH_ERR_OOM: return "out of memory";
    case BH_ERR_DEVICE: return "CUDA device error";
    case BH_ERR_OVERFLOW_STACK: return "tree-walk stack overflow";
    case BH_ERR_OVERFLOW_HASH: return "node hash table overflow";
    case BH_ERR_OVERFLOW_NODES: return "node arena overflow";
    case BH_ERR_TIMEOUT: return "device wait timed out";
    case BH_ERR_NO_TREE: return "no tree has been built";
    case BH_ERR_NOT_FOUND: return "node not found";
  }
  return "unknown status";
}

void bh_params_default(bh_params* p) {
  if (!p) return;
  p->theta = 0.5;
  p->eps = 0.025;
  p->dt = 1e-3;
  p->leaf_capacity = 1;
  p->multipole = BH_MULTIPOLE_QUADRUPOLE;
  p->edge_factor = 2.0;
  p->acc_follows_body = 1;
}

bh_status bh_destroy(bh_ctx* c) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->stage_ev)
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < 2; ++k) {
    dfree(c->pos[k]);
    dfree(c->vel[k]);
    dfree(c->keys[k]);
    dfree(c->vals[k]);
  }
  dfree(c->acc);
  dfree(c->body_key);
  dfree(c->tkey);
  dfree(c->tslot);
  dfree(c->tpos);
  dfree(c->sort.hist);
  dfree(c->sort.lookback);
  dfree(c->sort.tile_ctr);
  dfree(c->nkey);
  dfree(c->nrange);
  dfree(c->wnode);
  dfree(c->nup);
  dfree(c->nchildbyte);
  dfree(c->nparent);
  dfree(c->narrived);
  dfree(c->lb_level);
  dfree(c->level_bounds);
  dfree(c->level_tile_ctr);
  dfree(c->hash_keys);
  dfree(c->hash_vals);
  for (auto& g : c->graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& g : c->host_graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& e : c->io_ev)
    if (e) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  bh::adj_release(c);
  dfree(c->sys_off);
  dfree(c->sys_geom);
  dfree(c->body_sys);
  dfree(c->groups);
  dfree(c->geom);
  dfree(c->bounds_partial);
  dfree(c->err);
  dfree(c->counters);
  if (c->flush_buf) cudaFree(c->flush_buf);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->h_counters) cudaFreeHost(c->h_counters);
  if (c->h_level_bounds) cudaFreeHost(c->h_level_bounds);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return BH_OK;
}

bh_status bh_create(bh_ctx** out, size_t capacity, int device) {
  if (!out || capacity == 0 || capacity > kMaxBodies) return BH_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) {
    cudaGetLastError();
    return BH_ERR_DEVICE;
  }
  if (cudaSetDevice(device) != cudaSuccess) return BH_ERR_DEVICE;
  bh::sort_init();
  bh::walk_init();
  bh::tree_init();
  bh_ctx* c = new (std::nothrow) bh_ctx();
  if (!c) return BH_ERR_OOM;
  c->device = device;
  c->cap = capacity;
  if (cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || c->sms <= 0) {
    cudaGetLastError();
    delete c;
    return BH_ERR_DEVICE;
  }
  auto fail = [&](bh_status s) {
    bh_destroy(c);
    return s;
  };
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) return fail(BH_ERR_DEVICE);
  c->stream = c->own_stream;
  for (auto& e : c->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(BH_ERR_DEVICE);
  for (auto& e : c->stage_ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(BH_ERR_DEVICE);
  bh_status s = BH_OK;
  for (int k = 0; k < 2 && s == BH_OK; ++k) {
    if ((s = dalloc(&c->pos[k], capacity)) != BH_OK) break;
    if ((s = dalloc(&c->vel[k], capacity)) != BH_OK) break;
    if ((s = dalloc(&c->keys[k], capacity)) != BH_OK) break;
    s = dalloc(&c->vals[k], capacity);
  }
  if (s == BH_OK) s = dalloc(&c->acc, capacity);
  if (s == BH_OK) s = dalloc(&c->body_key, capacity);
  if (s == BH_OK) s = dalloc(&c->tkey, capacity);
  if (s == BH_OK) s = dalloc(&c->tslot, capacity);
  if (s == BH_OK) s = dalloc(&c->tpos, capacity);
  c->sort.max_tiles = bh::sort_max_tiles(capacity);
  if (s == BH_OK) s = dalloc(&c->sort.hist, 8 * 256);
  if (s == BH_OK) s = dalloc(&c->sort.lookback, (size_t)8 * c->sort.max_tiles * 256);
  if (s == BH_OK) s = dalloc(&c->sort.tile_ctr, 8);
  // tiles per level: 256 nodes each, or 8 each on the levels built one warp per node
  c->lb_level_tiles = (int)std::max<size_t>((capacity + 255) / 256 + 1, kLevelWarpNodes / 8 + 1);
  if (s == BH_OK) s = dalloc(&c->lb_level, (size_t)kLevels * c->lb_level_tiles);
  if (s == BH_OK) s = dalloc(&c->level_bounds, kLevels + 2);
  if (s == BH_OK) s = dalloc(&c->level_tile_ctr, kLevels);
  if (s == BH_OK) s = dalloc(&c->geom, 1);
  c->bounds_blocks = c->sms * 2;
  if (s == BH_OK) s = dalloc(&c->bounds_partial, (size_t)c->bounds_blocks * 6);
  if (s == BH_OK) s = dalloc(&c->err, 1);
  if (s == BH_OK) s = dalloc(&c->counters, 1);
  if (s != BH_OK) return fail(s);
  if (cudaMallocHost((void**)&c->h_err, sizeof(uint32_t)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_counters, sizeof(bh::Counters)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_level_bounds, sizeof(int) * (kLevels + 2)) != cudaSuccess)
    return fail(BH_ERR_OOM);
  cudaMemsetAsync(c->err, 0, sizeof(uint32_t), c->stream);
  cudaMemsetAsync(c->counters, 0, sizeof(bh::Counters), c->stream);
  cudaMemsetAsync(c->acc, 0, sizeof(float4) * capacity, c->stream);
  cudaMemsetAsync(c->body_key, 0, sizeof(uint64_t) * capacity, c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(BH_ERR_DEVICE);
  *out = c;
  return BH_OK;
}

bh_status bh_num_bodies(const bh_ctx* c, size_t* n) {
  if (!c || !n) return BH_ERR_INVALID_ARG;
  *n = c->n;
  return BH_OK;
}

bh_status bh_set_state(bh_ctx* c, const float* pos_m4, const float* vel4, const float* acc4, size_t n) {
  if (!c || n > c->cap || (n > 0 && (!pos_m4 || !vel4))) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  bh::reset_state(c, n);
  if (n > 0) {
    cudaMemcpyAsync(c->pos[0], pos_m4, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->vel[0], vel4, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream);
    if (acc4) cudaMemcpyAsync(c->acc, acc4, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream);
  }
  return cuda_status(cudaStreamSynchronize(c->stream));
}

bh_status bh_set_bodies(bh_ctx* c, const float* pos_m4, const float* vel4, size_t n) {
  return bh_set_state(c, pos_m4, vel4, nullptr, n);
}

bh_status bh_get_bodies(bh_ctx* c, float* pos_m4, float* vel4, float* acc4) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  const size_t n = c->n;
  if (n > 0) {
    if (pos_m4) cudaMemcpyAsync(pos_m4, c->pos[c->cur], sizeof(float4) * n, cudaMemcpyDeviceToHost, c->stream);
    if (vel4) cudaMemcpyAsync(vel4, c->vel[c->cur], sizeof(float4) * n, cudaMemcpyDeviceToHost, c->stream);
    if (acc4) cudaMemcpyAsync(acc4, c->acc, sizeof(float4) * n, cudaMemcpyDeviceToHost, c->stream);
  }
  return cuda_status(cudaStreamSynchronize(c->stream));
}

// Reference Body layout (80 bytes): ofColor@0, displayRadius@8, position@16, velocity@40,
// mass@64, bodyKey@72.
bh_status bh_set_bodies_ref(bh_ctx* c, const void* bodies, size_t n) {
  if (!c || n > c->cap || (n > 0 && !bodies)) return BH_ERR_INVALID_ARG;
  std::vector<float> p(4 * n), v(4 * n);
  const unsigned char* b = (const unsigned char*)bodies;
  for (size_t i = 0; i < n; ++i) {
    double rec[8];
    std::memcpy(rec, b + 80 * i + 16, 7 * sizeof(double));
    for (int k = 0; k < 3; ++k) {
      p[4 * i + k] = (float)rec[k];
      v[4 * i + k] = (float)rec[3 + k];
    }
    p[4 * i + 3] = (float)rec[6];
    v[4 * i + 3] = 0.f;
  }
  return bh_set_bodies(c, p.data(), v.data(), n);
}

bh_status bh_get_bodies_ref(bh_ctx* c, void* bodies, size_t n) {
  if (!c || !bodies || n != c->n) return BH_ERR_INVALID_ARG;
  std::vector<float> p(4 * n), v(4 * n);
  std::vector<uint64_t> k(n);
  BH_TRY(bh_get_bodies(c, p.data(), v.data(), nullptr));
  if (n > 0) {
    cudaMemcpy(k.data(), c->body_key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost);
    BH_TRY(last_launch());
  }
  unsigned char* b = (unsigned char*)bodies;
  for (size_t i = 0; i < n; ++i) {
    double rec[7] = {p[4 * i], p[4 * i + 1], p[4 * i + 2], v[4 * i], v[4 * i + 1], v[4 * i + 2], p[4 * i + 3]};
    std::memcpy(b + 80 * i + 16, rec, sizeof(rec));
    std::memcpy(b + 80 * i + 72, &k[i], sizeof(uint64_t));
  }
  return BH_OK;
}

bh_status bh_compute_bounds(bh_ctx* c, bh_bounds* out) {
  if (!c || !out) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  bh::launch_bounds(c, c->pos[c->cur], (int)c->n, 1.0);
  BH_TRY(last_launch());
  bh::Geom g;
  cudaMemcpyAsync(&g, c->geom, sizeof(g), cudaMemcpyDeviceToHost, c->stream);
  BH_TRY(cuda_status(cudaStreamSynchronize(c->stream)));
  for (int a = 0; a < 3; ++a) out->center[a] = g.center[a];
  out->size = g.size;
  return BH_OK;
}

bh_status bh_morton_keys(bh_ctx* c, double size, uint64_t* keys_out) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  const int n = (int)c->n;
  const double zero[3] = {0, 0, 0};
  bh::launch_set_geom(c, zero, size, zero, 1.0);
  bh::launch_morton(c, c->pos[c->cur], n, c->body_key, c->vals[0]);
  BH_TRY(last_launch());
  if (keys_out && n > 0)
    cudaMemcpyAsync(keys_out, c->body_key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, c->stream);
  return cuda_status(cudaStreamSynchronize(c->stream));
}

bh_status bh_decode_morton_keys(bh_ctx* c, const uint64_t* keys, size_t n, double size, double* pos3_out) {
  if (!c || (n > 0 && (!keys || !pos3_out)) || n > (size_t)INT32_MAX) return BH_ERR_INVALID_ARG;
  if (n == 0) return BH_OK;
  cudaSetDevice(c->device);
  uint64_t* dk = nullptr;
  double* dp = nullptr;
  BH_TRY(dalloc(&dk, n));
  bh_status s = dalloc(&dp, 3 * n);
  if (s == BH_OK) {
    cudaMemcpyAsync(dk, keys, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, c->stream);
    bh::launch_decode_morton(c, dk, (int)n, size, dp);
    s = last_launch();
    if (s == BH_OK) cudaMemcpyAsync(pos3_out, dp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream);
    if (s == BH_OK) s = cuda_status(cudaStreamSynchronize(c->stream));
  }
  dfree(dk);
  dfree(dp);
  return s;
}

bh_status bh_sort_bodies(bh_ctx* c, uint32_t* perm_out) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  const int n = (int)c->n;
  if (n == 0) return BH_OK;
  clear_device_flags(c);
  c->launches += 1;
  k_iota<<<(n + 255) / 256, 256, 0, c->stream>>>(c->vals[0], n);
  uint64_t* ko;
  uint32_t* vo;
  bh::radix_sort_pairs(c, c->body_key, c->vals[0], c->keys[1], c->vals[1], n, c->stream, &ko, &vo);
  const int nx = 1 - c->cur;
  bh::launch_gather(c, vo, n, c->pos[c->cur], c->vel[c->cur], c->pos[nx], c->vel[nx]);
  BH_TRY(last_launch());
  if (perm_out) cudaMemcpyAsync(perm_out, vo, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, c->stream);
  uint32_t e = 0;
  BH_TRY(sync_and_check(c, &e));
  if (e) return err_to_status(e);
  c->cur = nx;
  c->tree_valid = false;
  c->hash_valid = false;
  return BH_OK;
}

bh_status bh_build(bh_ctx* c, const double center[3], double edge, int leaf_capacity, int multipole) {
  bh::Range range_("bh_build");
  if (!c || !center || !(edge > 0) || leaf_capacity < 1 ||
      (multipole != BH_MULTIPOLE_LITERAL && multipole != BH_MULTIPOLE_QUADRUPOLE))
    return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  const int n = (int)c->n;
  BH_TRY(ensure_nodes(c, initial_node_cap(c->n)));
  for (;;) {
    clear_device_flags(c);
    bh::launch_set_geom(c, center, edge, center, edge);
    enqueue_tree(c, c->pos[c->cur], n, leaf_capacity, multipole, false);
    bh::launch_build(c, n, leaf_capacity);
    bh::launch_upsweep(c, n, leaf_capacity, multipole);
    BH_TRY(last_launch());
    uint32_t e = 0;
    BH_TRY(sync_and_check(c, &e));
    if (e & bh::kErrNodes) {
      BH_TRY(ensure_nodes(c, c->node_cap * 2));
      continue;
    }
    if (e) return err_to_status(e);
    break;
  }
  c->tree_valid = true;
  c->hash_valid = false;  // rebuilt on the first lookup after a build
  c->tree_leaf_cap = leaf_capacity;
  c->tree_mode = multipole;
  for (int a = 0; a < 3; ++a) c->tree_center[a] = center[a];
  c->tree_edge = edge;
  return BH_OK;
}

bh_status bh_tree_size(bh_ctx* c, size_t* m) {
  if (!c || !m) return BH_ERR_INVALID_ARG;
  if (!c->tree_valid) return BH_ERR_NO_TREE;
  *m = c->n ? (size_t)c->h_level_bounds[kLevels] : 0;
  return BH_OK;
}

bh_status bh_tree_nodes(bh_ctx* c, size_t cap, uint64_t* keys, int64_t* counts, double* mass, double* com3,
                        uint8_t* child_byte, double* quad6) {
  if (!c) return BH_ERR_INVALID_ARG;
  if (!c->tree_valid) return BH_ERR_NO_TREE;
  size_t m = 0;
  BH_TRY(bh_tree_size(c, &m));
  if (cap < m) return BH_ERR_INVALID_ARG;
  if (m == 0) return BH_OK;
  cudaSetDevice(c->device);
  std::vector<int2> r(m);
  std::vector<bh::NodeUp> f(m);
  if (keys) cudaMemcpyAsync(keys, c->nkey, sizeof(uint64_t) * m, cudaMemcpyDeviceToHost, c->stream);
  if (child_byte) cudaMemcpyAsync(child_byte, c->nchildbyte, m, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(r.data(), c->nrange, sizeof(int2) * m, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(f.data(), c->nup, sizeof(bh::NodeUp) * m, cudaMemcpyDeviceToHost, c->stream);
  BH_TRY(cuda_status(cudaStreamSynchronize(c->stream)));
  for (size_t j = 0; j < m; ++j) {
    if (counts) counts[j] = r[j].y;
    if (mass) mass[j] = (double)f[j].mass_hi + (double)f[j].mass_lo;
    if (com3)
      for (int a = 0; a < 3; ++a) com3[3 * j + a] = (double)f[j].com_hi[a] + (double)f[j].com_lo[a];
    if (quad6)
      for (int k = 0; k < 6; ++k) quad6[6 * j + k] = f[j].q[k];
  }
  return BH_OK;
}

bh_status bh_node_lookup(bh_ctx* c, uint64_t key, bh_node* out) {
  if (!c || !out) return BH_ERR_INVALID_ARG;
  if (!c->tree_valid) return BH_ERR_NO_TREE;
  cudaSetDevice(c->device);
  if (!c->hash_valid) {
    BH_TRY(ensure_hash(c));
    clear_device_flags(c);
    bh::launch_hash(c);
    uint32_t e = 0;
    BH_TRY(sync_and_check(c, &e));
    if (e) return err_to_status(e);
    c->hash_valid = true;
  }
  int* d_idx = nullptr;
  BH_TRY(dalloc(&d_idx, 1));
  bh::launch_lookup(c, key, d_idx);
  int idx = -1;
  cudaMemcpyAsync(&idx, d_idx, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  dfree(d_idx);
  BH_TRY(last_launch());
  if (idx < 0) return BH_ERR_NOT_FOUND;
  int2 r;
  bh::NodeUp f;
  uint8_t cb = 0;
  cudaMemcpy(&r, c->nrange + idx, sizeof(r), cudaMemcpyDeviceToHost);
  cudaMemcpy(&f, c->nup + idx, sizeof(f), cudaMemcpyDeviceToHost);
  cudaMemcpy(&cb, c->nchildbyte + idx, 1, cudaMemcpyDeviceToHost);
  BH_TRY(last_launch());
  std::memset(out, 0, sizeof(*out));
  out->key = key;
  out->count = r.y;
  out->mass = (double)f.mass_hi + (double)f.mass_lo;
  for (int a = 0; a < 3; ++a) out->com[a] = (double)f.com_hi[a] + (double)f.com_lo[a];
  for (int k = 0; k < 6; ++k) out->quad[k] = f.q[k];
  out->child_byte = cb;
  // node bounds from the key, by the reference's child-centre recurrence
  int depth = 0;
  for (uint64_t k = key; k > 1; k >>= 3) ++depth;
  double cc[3] = {c->tree_center[0], c->tree_center[1], c->tree_center[2]}, s = c->tree_edge;
  for (int d = depth - 1; d >= 0; --d) {
    int o = (int)((key >> (3 * d)) & 7);
    double half = s * 0.5;
    for (int a = 0; a < 3; ++a) {
      volatile double off = (((o >> (2 - a)) & 1) ? 0.5 : -0.5) * half;
      cc[a] = cc[a] + off;
    }
    s = half;
  }
  for (int a = 0; a < 3; ++a) out->center[a] = cc[a];
  out->size = s;
  out->depth = depth;
  return BH_OK;
}

bh_status bh_force(bh_ctx* c, double theta, double eps, float* acc4_out, bh_stats* st) {
  bh::Range range_("bh_force");
  if (!c || !(theta >= 0) || !(eps >= 0)) return BH_ERR_INVALID_ARG;
  if (!c->tree_valid) return BH_ERR_NO_TREE;
  cudaSetDevice(c->device);
  const int n = (int)c->n;
  clear_device_flags(c);
  record(c, st, 0);
  bh::launch_walk(c, n, (float)theta, (float)eps, c->tree_mode, c->acc, nullptr, 0.f);
  record(c, st, 1);
  BH_TRY(last_launch());
  if (acc4_out && n > 0)
    cudaMemcpyAsync(acc4_out, c->acc, sizeof(float4) * n, cudaMemcpyDeviceToHost, c->stream);
  uint32_t e = 0;
  BH_TRY(sync_and_check(c, &e));
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->ms_walk = elapsed(c, 0, 1);
    st->ms_step = st->ms_walk;
    st->interactions_cell = c->h_counters->cell;
    st->interactions_p2p = c->h_counters->p2p;
    st->walk_cell_evals = c->h_counters->cell_evals;
    st->walk_point_evals = c->h_counters->point_evals;
    st->n_nodes = (uint64_t)c->h_level_bounds[kLevels];
    st->error_flags = e;
    st->kernel_launches = 1;
  }
  return err_to_status(e);
}

bh_status bh_kick_drift(bh_ctx* c, double dt) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  bh::launch_kick_drift(c, c->pos[c->cur], c->vel[c->cur], c->acc, (int)c->n, (float)dt, 1);
  BH_TRY(last_launch());
  c->tree_valid = false;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

bh_status bh_kick(bh_ctx* c, double dt) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  bh::launch_kick_drift(c, c->pos[c->cur], c->vel[c->cur], c->acc, (int)c->n, (float)dt, 0);
  BH_TRY(last_launch());
  return cuda_status(cudaStreamSynchronize(c->stream));
}

}  // extern "C"

namespace {

// Host buffers of bh_step_host (pinned; any may be null). vel_out_dev is vel_out's address in
// the device's address space when the buffer is mapped and 16-byte aligned: the walk's kick then
// writes the velocities there itself and no download follows the walk.
struct HostIO {
  const float* pos_in;
  const float* vel_in;
  float* pos_out;
  float* vel_out;
  float4* vel_out_dev;
};

// Device address of a pinned host buffer for direct float4 stores, or null (not mapped, or not
// 16-byte aligned).
float4* mapped_float4(void* host) {
  if (!host) return nullptr;
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, host, 0) != cudaSuccess || !d) {
    cudaGetLastError();
    return nullptr;
  }
  return (reinterpret_cast<uintptr_t>(d) % alignof(float4)) == 0 ? static_cast<float4*>(d) : nullptr;
}

bh_status ensure_copy_stream(bh_ctx* c);  // the second stream of the *_step_host calls

// Step graphs are captured on the context's own stream (a caller's stream may be one that
// cannot be captured, such as the legacy default stream) and launched on c->stream; the guard
// points c->stream at the own stream for the capture and restores it on every exit.
struct CaptureOnOwnStream {
  bh_ctx* c;
  cudaStream_t saved;
  explicit CaptureOnOwnStream(bh_ctx* ctx) : c(ctx), saved(ctx->stream) { c->stream = c->own_stream; }
  ~CaptureOnOwnStream() { c->stream = saved; }
};

bool pinned(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// One plain step enqueued on c->stream without host synchronisation (capturable). Stage events
// are external event-record nodes when captured (a plain record during capture would only order
// the capture, not record the event). With io, the positions upload first, then the copies run
// on c->copy_stream beside the step: the velocities upload while bounds, keys and sort run; the
// positions, final after the drift, download while the tree is built and walked; the velocities
// download after the walk's kick.
void enqueue_plain_step(bh_ctx* c, const bh_params* prm, const HostIO* io, bool marks) {
  const int n = (int)c->n, cur = c->cur, nx = 1 - cur;
  const float dt = (float)prm->dt;
  const size_t bytes = sizeof(float4) * (size_t)n;
  auto mark = [&](int k) {
    if (marks) cudaEventRecordWithFlags(c->stage_ev[k], c->stream, cudaEventRecordExternal);
  };
  if (io) {
    // positions first, alone on the link (the bounds wait for them); the velocities follow on
    // the second stream beside bounds, keys and sort (two uploads at once would share the
    // link's bandwidth and delay the positions)
    if (io->pos_in) cudaMemcpyAsync(c->pos[cur], io->pos_in, bytes, cudaMemcpyHostToDevice, c->stream);
    cudaEventRecord(c->io_ev[0], c->stream);  // fork
    cudaStreamWaitEvent(c->copy_stream, c->io_ev[0], 0);
    if (io->vel_in) cudaMemcpyAsync(c->vel[cur], io->vel_in, bytes, cudaMemcpyHostToDevice, c->copy_stream);
    cudaEventRecord(c->io_ev[1], c->copy_stream);
  }
  clear_device_flags(c);
  mark(0);
  bh::launch_bounds(c, c->pos[cur], n, prm->edge_factor);
  mark(1);
  bh::launch_morton(c, c->pos[cur], n, c->keys[0], c->vals[0]);
  mark(2);
  uint64_t* ko;
  uint32_t* perm;
  bh::radix_sort_pairs(c, c->keys[0], c->vals[0], c->keys[1], c->vals[1], n, c->stream, &ko, &perm);
  mark(3);
  if (io) cudaStreamWaitEvent(c->stream, c->io_ev[1], 0);
  bh::launch_gather_kd_treekey(c, perm, n, c->pos[cur], c->vel[cur], c->acc, prm->acc_follows_body, dt, c->pos[nx],
                               c->vel[nx], c->tkey, c->tslot);
  mark(4);
  if (io) {
    cudaEventRecord(c->io_ev[2], c->stream);
    cudaStreamWaitEvent(c->copy_stream, c->io_ev[2], 0);
    if (io->pos_out) cudaMemcpyAsync(io->pos_out, c->pos[nx], bytes, cudaMemcpyDeviceToHost, c->copy_stream);
    cudaEventRecord(c->io_ev[3], c->copy_stream);
  }
  enqueue_tree(c, c->pos[nx], n, prm->leaf_capacity, prm->multipole, true);
  mark(5);
  bh::launch_build(c, n, prm->leaf_capacity);
  mark(6);
  bh::launch_upsweep(c, n, prm->leaf_capacity, prm->multipole);
  mark(7);
  float4* vel_copy = io ? io->vel_out_dev : nullptr;
  bh::launch_walk(c, n, (float)prm->theta, (float)prm->eps, prm->multipole, c->acc, c->vel[nx], 0.5f * dt, false,
                  vel_copy);
  mark(8);
  if (io) {
    if (io->vel_out && !vel_copy)
      cudaMemcpyAsync(io->vel_out, c->vel[nx], bytes, cudaMemcpyDeviceToHost, c->stream);
    cudaStreamWaitEvent(c->stream, c->io_ev[3], 0);  // join
  }
}

bool same_io(const HostIO& a, const void* const b[4]) {
  return a.pos_in == b[0] && a.vel_in == b[1] && a.pos_out == b[2] && a.vel_out == b[3];
}

// Runs nsteps plain steps, each one replay of a CUDA graph captured per state parity on first use
// (the step's ~70 launches cost one graph launch). io (one step only) selects the graphs that
// carry the host copies, captured per set of host buffers.
bh_status run_plain_steps(bh_ctx* c, const bh_params* prm, int nsteps, bh_stats* st, const HostIO* io) {
  BH_TRY(ensure_nodes(c, initial_node_cap(c->n)));
  const bool marks = st != nullptr;  // stage events only for calls that return their times
  const uint64_t launches0 = c->launches;
  if (!same_params(c->graph_params, *prm)) destroy_graphs(c);
  c->graph_params = *prm;
  for (int s = 0; s < nsteps; ++s) {
    uint32_t e = 0;
    for (;;) {
      const int par = c->cur;
      cudaGraphExec_t& graph = io ? c->host_graph[par] : c->graph[par];
      uint64_t*& keys0 = io ? c->host_graph_keys0[par] : c->graph_keys0[par];
      uint64_t& kernels = io ? c->host_graph_kernels[par] : c->graph_kernels[par];
      bool& gmarks = io ? c->host_graph_marks[par] : c->graph_marks[par];
      // captured with other key buffers (they swap every step), other host buffers, or with
      // stage events when these are (not) wanted now
      if (graph && (keys0 != c->keys[0] || gmarks != marks || (io && !same_io(*io, c->host_graph_ptrs[par])))) {
        cudaGraphExecDestroy(graph);
        graph = nullptr;
      }
      if (!graph) {
        CaptureOnOwnStream on_own(c);
        cudaGraph_t g = nullptr;
        BH_TRY(cuda_status(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal)));
        const uint64_t l0 = c->launches;
        enqueue_plain_step(c, prm, io, marks);
        gmarks = marks;
        kernels = c->launches - l0;  // counted when the graph runs, not when captured
        c->launches = l0;
        cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
        if (ce != cudaSuccess || !g) return cuda_status(ce == cudaSuccess ? cudaErrorUnknown : ce);
        ce = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
          graph = nullptr;
          return cuda_status(ce);
        }
        keys0 = c->keys[0];
        c->graph_n = c->n;
        if (io) {
          c->host_graph_ptrs[par][0] = io->pos_in;
          c->host_graph_ptrs[par][1] = io->vel_in;
          c->host_graph_ptrs[par][2] = io->pos_out;
          c->host_graph_ptrs[par][3] = io->vel_out;
        }
      }
      BH_TRY(cuda_status(cudaGraphLaunch(graph, c->stream)));
      c->launches += kernels;
      BH_TRY(last_launch());
      BH_TRY(sync_and_check(c, &e));
      if (e & bh::kErrNodes) {  // arena too small: grow it (dropping the graphs) and redo the step
        BH_TRY(ensure_nodes(c, c->node_cap * 2));
        if (st) st->retries++;
        continue;
      }
      break;
    }
    if (e) return err_to_status(e);
    // the sorted Morton keys become the bodies' keys (Body::bodyKey after RadixSortBodies)
    uint64_t* tmp = c->body_key;
    c->body_key = c->keys[0];
    c->keys[0] = tmp;
    c->cur = 1 - c->cur;
    c->tree_valid = true;
    c->tree_leaf_cap = prm->leaf_capacity;
    c->tree_mode = prm->multipole;
    if (st) {
      st->ms_step += elapsed(c, 0, 8);
      st->ms_bounds += elapsed(c, 0, 1);
      st->ms_morton += elapsed(c, 1, 2);
      st->ms_sort += elapsed(c, 2, 3);
      st->ms_kick_drift += elapsed(c, 3, 4);
      st->ms_sort_tree += elapsed(c, 4, 5);
      st->ms_build += elapsed(c, 5, 6);
      st->ms_upsweep += elapsed(c, 6, 7);
      st->ms_walk += elapsed(c, 7, 8);
      st->n_nodes = (uint64_t)c->h_level_bounds[kLevels];
      st->interactions_cell += c->h_counters->cell;
      st->interactions_p2p += c->h_counters->p2p;
      st->walk_cell_evals += c->h_counters->cell_evals;
      st->walk_point_evals += c->h_counters->point_evals;
      st->max_depth = std::max(st->max_depth, c->h_counters->max_depth);
      st->steps++;
    }
  }
  if (st) st->kernel_launches = (uint32_t)(c->launches - launches0);
  // tree geometry of the last step, for node lookups
  bh::Geom g;
  cudaMemcpy(&g, c->geom, sizeof(g), cudaMemcpyDeviceToHost);
  for (int a = 0; a < 3; ++a) c->tree_center[a] = g.tc[a];
  c->tree_edge = g.tedge;
  c->hash_valid = false;
  return last_launch();
}

bool valid_params(const bh_params* prm) {
  return prm && prm->leaf_capacity >= 1 && prm->theta >= 0 && prm->eps >= 0 && prm->edge_factor > 0 &&
         (prm->multipole == BH_MULTIPOLE_LITERAL || prm->multipole == BH_MULTIPOLE_QUADRUPOLE);
}

}  // namespace

extern "C" {

bh_status bh_step(bh_ctx* c, const bh_params* prm, int nsteps, bh_stats* st) {
  bh::Range range_("bh_step");
  if (!c || nsteps < 0 || !valid_params(prm)) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (st) std::memset(st, 0, sizeof(*st));
  if (c->n == 0 || nsteps == 0) return BH_OK;
  return run_plain_steps(c, prm, nsteps, st, nullptr);
}

bh_status bh_step_host(bh_ctx* c, const bh_params* prm, const float* pos_m4_in, const float* vel4_in,
                       float* pos_m4_out, float* vel4_out, bh_stats* st) {
  bh::Range range_("bh_step_host");
  if (!c || !valid_params(prm)) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (st) std::memset(st, 0, sizeof(*st));
  if (c->n == 0) return BH_OK;
  const HostIO io{pos_m4_in, vel4_in, pos_m4_out, vel4_out, mapped_float4(vel4_out)};
  if (!(pinned(pos_m4_in) && pinned(vel4_in) && pinned(pos_m4_out) && pinned(vel4_out))) {
    // pageable buffers cannot be captured: copy, step, copy in order on the context's stream
    const size_t bytes = sizeof(float4) * c->n;
    if (pos_m4_in) cudaMemcpyAsync(c->pos[c->cur], pos_m4_in, bytes, cudaMemcpyHostToDevice, c->stream);
    if (vel4_in) cudaMemcpyAsync(c->vel[c->cur], vel4_in, bytes, cudaMemcpyHostToDevice, c->stream);
    BH_TRY(run_plain_steps(c, prm, 1, st, nullptr));
    return bh_get_bodies(c, pos_m4_out, vel4_out, nullptr);
  }
  BH_TRY(ensure_copy_stream(c));
  return run_plain_steps(c, prm, 1, st, &io);
}

bh_status bh_synchronize(bh_ctx* c) {
  if (!c) return BH_ERR_INVALID_ARG;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

bh_status bh_set_stream(bh_ctx* c, void* stream) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  BH_TRY(cuda_status(cudaStreamSynchronize(c->stream)));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return BH_OK;
}

bh_status bh_get_stream(bh_ctx* c, void** stream_out, int* device_out) {
  if (!c) return BH_ERR_INVALID_ARG;
  if (stream_out) *stream_out = (void*)c->stream;
  if (device_out) *device_out = c->device;
  return BH_OK;
}

bh_status bh_event_record(bh_ctx* c, int slot) {
  if (!c || slot < 0 || slot >= bh::kNumEvents) return BH_ERR_INVALID_ARG;
  return cuda_status(cudaEventRecord(c->ev[slot], c->stream));
}

bh_status bh_event_elapsed_ms(bh_ctx* c, int a, int b, float* ms) {
  if (!c || !ms || a < 0 || b < 0 || a >= bh::kNumEvents || b >= bh::kNumEvents) return BH_ERR_INVALID_ARG;
  BH_TRY(cuda_status(cudaEventSynchronize(c->ev[b])));
  return cuda_status(cudaEventElapsedTime(ms, c->ev[a], c->ev[b]));
}

bh_status bh_flush_l2(bh_ctx* c) {
  if (!c) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (!c->flush_buf) {
    c->flush_bytes = (size_t)512 << 20;
    if (cudaMalloc(&c->flush_buf, c->flush_bytes) != cudaSuccess) {
      cudaGetLastError();
      c->flush_buf = nullptr;
      return BH_ERR_OOM;
    }
  }
  static int salt = 0;
  return cuda_status(cudaMemsetAsync(c->flush_buf, (++salt) & 0xff, c->flush_bytes, c->stream));
}

bh_status bh_host_alloc(void** ptr, size_t bytes) {
  if (!ptr) return BH_ERR_INVALID_ARG;
  if (cudaMallocHost(ptr, bytes ? bytes : 1) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return BH_ERR_OOM;
  }
  return BH_OK;
}

bh_status bh_host_free(void* ptr) {
  if (ptr) cudaFreeHost(ptr);
  return BH_OK;
}

bh_status bh_measure_fp32_peak(bh_ctx* c, double* tflops) {
  if (!c || !tflops) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  float* sink = nullptr;
  BH_TRY(dalloc(&sink, 1));
  const int blocks = sms * 8;
  bh::launch_fp32_peak(c->stream, sink, blocks);  // warm-up
  cudaEventRecord(c->ev[bh::kNumEvents - 2], c->stream);
  bh::launch_fp32_peak(c->stream, sink, blocks);
  cudaEventRecord(c->ev[bh::kNumEvents - 1], c->stream);
  float ms = 0;
  cudaEventSynchronize(c->ev[bh::kNumEvents - 1]);
  cudaEventElapsedTime(&ms, c->ev[bh::kNumEvents - 2], c->ev[bh::kNumEvents - 1]);
  dfree(sink);
  BH_TRY(last_launch());
  const double flops = (double)blocks * 256 * 4096 * 16 * 8 * 2;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return BH_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Batched ensembles: many independent systems in one context, stepped together. Each system
// keeps a fixed body range [off[s], off[s+1]); every stage runs over all bodies at once:
// per-system bounds; Morton keys with the system's own cube; a stable sort by key followed by
// a stable sort by system id, which regroups every system in key order inside its range; the
// same for tree keys; one tree level build for all systems together (one root per system);
// one walk over groups of up to 32 bodies that never straddle a system, pulled from a global
// work queue. Each step is captured once per state parity in a CUDA graph and replayed.
// ---------------------------------------------------------------------------------------
namespace {

constexpr size_t kMaxSystems = 65535;  // system ids are stored as u16

void destroy_graphs(bh_ctx* c) {
  for (int k = 0; k < 2; ++k)
    for (cudaGraphExec_t* g : {&c->graph[k], &c->host_graph[k]})
      if (*g) {
        cudaGraphExecDestroy(*g);
        *g = nullptr;
      }
}

bool same_params(const bh_params& a, const bh_params& b) {
  return a.theta == b.theta && a.eps == b.eps && a.dt == b.dt && a.leaf_capacity == b.leaf_capacity &&
         a.multipole == b.multipole && a.edge_factor == b.edge_factor && a.acc_follows_body == b.acc_follows_body;
}

// One batched step, enqueued on c->stream without host synchronisation (capturable).
void enqueue_batch_step(bh_ctx* c, const bh_params& p, const HostIO* io, bool marks) {
  const int n = (int)c->n, cur = c->cur, nx = 1 - cur;
  const float dt = (float)p.dt;
  const size_t bytes = sizeof(float4) * (size_t)n;
  if (io) {  // the copies of bh_batch_step_host, beside the step as in enqueue_plain_step
    if (io->pos_in) cudaMemcpyAsync(c->pos[cur], io->pos_in, bytes, cudaMemcpyHostToDevice, c->stream);
    cudaEventRecord(c->io_ev[0], c->stream);
    cudaStreamWaitEvent(c->copy_stream, c->io_ev[0], 0);
    if (io->vel_in) cudaMemcpyAsync(c->vel[cur], io->vel_in, bytes, cudaMemcpyHostToDevice, c->copy_stream);
    cudaEventRecord(c->io_ev[1], c->copy_stream);
  }
  // stage events as in the plain step (external event-record nodes in the captured graph)
  auto mark = [&](int k) {
    if (marks) cudaEventRecordWithFlags(c->stage_ev[k], c->stream, cudaEventRecordExternal);
  };
  clear_device_flags(c);
  mark(0);
  bh::launch_batch_bounds(c, c->pos[c->cur], p.edge_factor);
  mark(1);
  bh::launch_morton(c, c->pos[c->cur], n, c->keys[0], c->vals[0], true);
  mark(2);
  uint64_t* ko;
  uint32_t* vo;
  bh::radix_sort_pairs(c, c->keys[0], c->vals[0], c->keys[1], c->vals[1], n, c->stream, &ko, &vo);
  bh::launch_sys_keys(c, c->vals[0], n, c->keys[1]);
  bh::radix_sort_pairs(c, c->keys[1], c->vals[0], c->keys[0], c->vals[1], n, c->stream, &ko, &vo, 0, 2);
  mark(3);
  // vals[0]: (system, Morton key) order; keys[0] receives the per-slot tree keys
  if (io) cudaStreamWaitEvent(c->stream, c->io_ev[1], 0);
  bh::launch_gather_kd_treekey(c, c->vals[0], n, c->pos[cur], c->vel[cur], c->acc, p.acc_follows_body, dt,
                               c->pos[nx], c->vel[nx], c->keys[0], c->tslot, true);
  mark(4);
  if (io) {
    cudaEventRecord(c->io_ev[2], c->stream);
    cudaStreamWaitEvent(c->copy_stream, c->io_ev[2], 0);
    if (io->pos_out) cudaMemcpyAsync(io->pos_out, c->pos[nx], bytes, cudaMemcpyDeviceToHost, c->copy_stream);
    cudaEventRecord(c->io_ev[3], c->copy_stream);
  }
  cudaMemcpyAsync(c->tkey, c->keys[0], sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, c->stream);
  bh::radix_sort_pairs(c, c->tkey, c->tslot, c->keys[1], c->vals[1], n, c->stream, &ko, &vo);
  bh::launch_sys_keys(c, c->tslot, n, c->keys[1]);
  bh::radix_sort_pairs(c, c->keys[1], c->tslot, c->tkey, c->vals[1], n, c->stream, &ko, &vo, 0, 2);
  bh::launch_gather_tree_keys(c, c->tslot, n, c->pos[nx], c->keys[0], c->tpos, c->tkey);
  mark(5);
  bh::launch_build(c, n, p.leaf_capacity, true);
  mark(6);
  bh::launch_upsweep(c, n, p.leaf_capacity, p.multipole, true);
  mark(7);
  float4* vel_copy = io ? io->vel_out_dev : nullptr;
  bh::launch_walk(c, n, (float)p.theta, (float)p.eps, p.multipole, c->acc, c->vel[nx], 0.5f * dt, true, vel_copy);
  mark(8);
  if (io) {
    if (io->vel_out && !vel_copy)
      cudaMemcpyAsync(io->vel_out, c->vel[nx], bytes, cudaMemcpyDeviceToHost, c->stream);
    cudaStreamWaitEvent(c->stream, c->io_ev[3], 0);  // join
  }
}

}  // namespace

extern "C" {

bh_status bh_batch_set(bh_ctx* c, const float* pos_m4, const float* vel4, const uint32_t* sys_offsets,
                       size_t nsys) {
  if (!c || !sys_offsets || nsys == 0 || nsys > kMaxSystems || sys_offsets[0] != 0) return BH_ERR_INVALID_ARG;
  for (size_t s = 0; s < nsys; ++s)
    if (sys_offsets[s + 1] <= sys_offsets[s]) return BH_ERR_INVALID_ARG;  // every system has a body
  const size_t n = sys_offsets[nsys];
  if (n > c->cap) return BH_ERR_INVALID_ARG;
  BH_TRY(bh_set_state(c, pos_m4, vel4, nullptr, n));
  return bh::batch_layout(c, sys_offsets, nsys);
}

}  // extern "C"

namespace bh {

bh_status check_sys_offsets(const bh_ctx* c, const uint32_t* sys_offsets, size_t nsys) {
  if (!c || !sys_offsets || nsys == 0 || nsys > kMaxSystems || sys_offsets[0] != 0) return BH_ERR_INVALID_ARG;
  for (size_t s = 0; s < nsys; ++s)
    if (sys_offsets[s + 1] <= sys_offsets[s]) return BH_ERR_INVALID_ARG;  // every system has a body
  return sys_offsets[nsys] > c->cap ? BH_ERR_INVALID_ARG : BH_OK;
}

// Ensemble layout over the bodies already in the state: system ids per slot, walk groups that
// never straddle systems, per-system geometry storage.
bh_status batch_layout(bh_ctx* c, const uint32_t* sys_offsets, size_t nsys) {
  const size_t n = sys_offsets[nsys];
  cudaSetDevice(c->device);
  destroy_graphs(c);
  if (c->sys_cap < nsys) {
    dfree(c->sys_off);
    dfree(c->sys_geom);
    c->sys_cap = 0;
    BH_TRY(dalloc(&c->sys_off, nsys + 1));
    BH_TRY(dalloc(&c->sys_geom, nsys));
    c->sys_cap = nsys;
  }
  if (!c->body_sys) BH_TRY(dalloc(&c->body_sys, c->cap));
  std::vector<uint16_t> bs(n);
  std::vector<int4> groups;
  for (size_t s = 0; s < nsys; ++s) {
    const uint32_t b0 = sys_offsets[s], b1 = sys_offsets[s + 1];
    for (uint32_t i = b0; i < b1; ++i) bs[i] = (uint16_t)s;
    for (uint32_t g = b0; g < b1; g += 32) groups.push_back(make_int4((int)g, (int)std::min(32u, b1 - g), (int)s, (int)s));
  }
  dfree(c->groups);
  BH_TRY(dalloc(&c->groups, groups.size()));
  c->ngroups = (int)groups.size();
  cudaMemcpyAsync(c->sys_off, sys_offsets, sizeof(uint32_t) * (nsys + 1), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->body_sys, bs.data(), sizeof(uint16_t) * n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->groups, groups.data(), sizeof(int4) * groups.size(), cudaMemcpyHostToDevice, c->stream);
  BH_TRY(cuda_status(cudaStreamSynchronize(c->stream)));
  c->nsys = (int)nsys;
  c->batch = true;
  return BH_OK;
}

// A new state of n bodies in slot order 0..n-1: every derived structure (tree, ensemble layout,
// recorded trajectory) is dropped; accelerations and Morton keys are zeroed. The caller fills
// pos[0] / vel[0]. Captured plain-step graphs stay valid for the same body count (they hold
// only buffer pointers); as the two Morton key buffers are interchangeable while the keys are
// zeroed, they are paired the way the state-0 graph was captured, so a reset followed by a
// step replays that graph instead of capturing a new one.
void reset_state(bh_ctx* c, size_t n) {
  c->n = n;
  c->cur = 0;
  c->tree_valid = false;
  c->batch = false;
  c->batch_tree_ready = false;
  adj_invalidate(c);
  if (n != c->graph_n)
    destroy_graphs(c);
  else if (c->graph[0] && c->graph_keys0[0] == c->body_key)
    std::swap(c->body_key, c->keys[0]);
  if (n > 0) {
    cudaMemsetAsync(c->acc, 0, sizeof(float4) * n, c->stream);
    cudaMemsetAsync(c->body_key, 0, sizeof(uint64_t) * n, c->stream);
  }
}

}  // namespace bh

extern "C" {

}  // extern "C"

namespace {

// nsteps batched steps, each one replay of a graph captured per state parity; with io (one
// step) the graphs that carry the host copies, captured per set of host buffers.
bh_status run_batch_steps(bh_ctx* c, const bh_params* prm, int nsteps, bh_stats* st, const HostIO* io) {
  const size_t need = std::max<size_t>(2 * c->n + 64 * (size_t)c->nsys, 1024);
  if (c->node_cap < need) destroy_graphs(c);
  BH_TRY(ensure_nodes(c, need));
  if (!same_params(c->graph_params, *prm)) destroy_graphs(c);
  c->graph_params = *prm;
  const bool marks = st != nullptr;  // stage events only for calls that return their times
  const uint64_t launches0 = c->launches;
  for (int s = 0; s < nsteps; ++s) {
    uint32_t e = 0;
    for (;;) {
      const int par = c->cur;
      cudaGraphExec_t& graph = io ? c->host_graph[par] : c->graph[par];
      uint64_t*& keys0 = io ? c->host_graph_keys0[par] : c->graph_keys0[par];
      uint64_t& kernels = io ? c->host_graph_kernels[par] : c->graph_kernels[par];
      bool& gmarks = io ? c->host_graph_marks[par] : c->graph_marks[par];
      // a plain step's graph (it records its key buffer), other host buffers, or stage events
      // when these are (not) wanted now
      if (graph && (keys0 || gmarks != marks || (io && !same_io(*io, c->host_graph_ptrs[par])))) {
        cudaGraphExecDestroy(graph);
        graph = nullptr;
      }
      if (!graph) {
        CaptureOnOwnStream on_own(c);
        cudaGraph_t g = nullptr;
        BH_TRY(cuda_status(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal)));
        keys0 = nullptr;
        const uint64_t l0 = c->launches;
        enqueue_batch_step(c, *prm, io, marks);
        gmarks = marks;
        kernels = c->launches - l0;  // counted when the graph runs, not when captured
        c->launches = l0;
        cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
        if (ce != cudaSuccess || !g) return cuda_status(ce == cudaSuccess ? cudaErrorUnknown : ce);
        ce = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
          graph = nullptr;
          return cuda_status(ce);
        }
        if (io) {
          c->host_graph_ptrs[par][0] = io->pos_in;
          c->host_graph_ptrs[par][1] = io->vel_in;
          c->host_graph_ptrs[par][2] = io->pos_out;
          c->host_graph_ptrs[par][3] = io->vel_out;
        }
      }
      BH_TRY(cuda_status(cudaGraphLaunch(graph, c->stream)));
      c->launches += kernels;
      BH_TRY(sync_and_check(c, &e));
      if (e & bh::kErrNodes) {  // arena too small: grow it, re-capture, redo the step
        destroy_graphs(c);
        BH_TRY(ensure_nodes(c, c->node_cap * 2));
        if (st) st->retries++;
        continue;
      }
      break;
    }
    if (e) return err_to_status(e);
    c->cur = 1 - c->cur;
    if (st) {
      st->ms_step += elapsed(c, 0, 8);
      st->ms_bounds += elapsed(c, 0, 1);
      st->ms_morton += elapsed(c, 1, 2);
      st->ms_sort += elapsed(c, 2, 3);
      st->ms_kick_drift += elapsed(c, 3, 4);
      st->ms_sort_tree += elapsed(c, 4, 5);
      st->ms_build += elapsed(c, 5, 6);
      st->ms_upsweep += elapsed(c, 6, 7);
      st->ms_walk += elapsed(c, 7, 8);
      st->n_nodes = (uint64_t)c->h_level_bounds[kLevels];
      st->interactions_cell += c->h_counters->cell;
      st->interactions_p2p += c->h_counters->p2p;
      st->walk_cell_evals += c->h_counters->cell_evals;
      st->walk_point_evals += c->h_counters->point_evals;
      st->max_depth = std::max(st->max_depth, c->h_counters->max_depth);
      st->steps++;
    }
  }
  if (st) st->kernel_launches = (uint32_t)(c->launches - launches0);
  c->tree_valid = false;  // the ensemble's tree is not a single-system tree
  c->hash_valid = false;
  c->batch_tree_ready = nsteps > 0;
  return last_launch();
}

bh_status ensure_copy_stream(bh_ctx* c) {
  if (c->copy_stream) return BH_OK;
  if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) return BH_ERR_DEVICE;
  for (auto& e : c->io_ev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return BH_ERR_DEVICE;
  return BH_OK;
}

}  // namespace

extern "C" {

bh_status bh_batch_step(bh_ctx* c, const bh_params* prm, int nsteps, bh_stats* st) {
  bh::Range range_("bh_batch_step");
  if (!c || nsteps < 0 || !c->batch || !valid_params(prm)) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (st) std::memset(st, 0, sizeof(*st));
  if (c->n == 0 || nsteps == 0) return BH_OK;
  return run_batch_steps(c, prm, nsteps, st, nullptr);
}

bh_status bh_batch_step_host(bh_ctx* c, const bh_params* prm, const float* pos_m4_in, const float* vel4_in,
                             float* pos_m4_out, float* vel4_out, bh_stats* st) {
  bh::Range range_("bh_batch_step_host");
  if (!c || !c->batch || !valid_params(prm)) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (st) std::memset(st, 0, sizeof(*st));
  if (c->n == 0) return BH_OK;
  const HostIO io{pos_m4_in, vel4_in, pos_m4_out, vel4_out, mapped_float4(vel4_out)};
  if (!(pinned(pos_m4_in) && pinned(vel4_in) && pinned(pos_m4_out) && pinned(vel4_out))) {
    const size_t bytes = sizeof(float4) * c->n;
    if (pos_m4_in) cudaMemcpyAsync(c->pos[c->cur], pos_m4_in, bytes, cudaMemcpyHostToDevice, c->stream);
    if (vel4_in) cudaMemcpyAsync(c->vel[c->cur], vel4_in, bytes, cudaMemcpyHostToDevice, c->stream);
    BH_TRY(run_batch_steps(c, prm, 1, st, nullptr));
    return bh_get_bodies(c, pos_m4_out, vel4_out, nullptr);
  }
  BH_TRY(ensure_copy_stream(c));
  return run_batch_steps(c, prm, 1, st, &io);
}

// Times every launch shape of the quadrupole walk on the tree in the arena (the last bh_step /
// bh_build, or the last bh_batch_step) and keeps the fastest for this context.
bh_status bh_autotune_walk(bh_ctx* c, double theta, double eps, int trials, bh_tune_result* out) {
  bh::Range range_("bh_autotune_walk");
  if (!c || !out || !(theta >= 0) || !(eps > 0) || trials < 1) return BH_ERR_INVALID_ARG;
  const bool batch = c->batch;
  if (batch ? !c->batch_tree_ready : !c->tree_valid) return BH_ERR_NO_TREE;
  cudaSetDevice(c->device);
  std::memset(out, 0, sizeof(*out));
  const int n = (int)c->n;
  const int nv = std::min(bh::walk_variants(), (int)BH_TUNE_MAX_VARIANTS);
  float4* scratch = nullptr;
  BH_TRY(dalloc(&scratch, c->n));
  bh_status status = BH_OK;
  float best_ms = 0.f;
  int best = 0;
  for (int v = 0; v < nv; ++v) {
    const bh::WalkVariant info = bh::walk_variant_info(v);
    out->warps_per_block[v] = info.warps;
    out->min_blocks_per_sm[v] = info.min_blocks;
    out->stack_depth[v] = info.stack;
    out->cell_form[v] = info.form;
    out->registers[v] = info.regs;
    out->group_size[v] = batch ? 32 : info.group;  // ensembles walk their fixed group table
    std::vector<float> ms;
    uint32_t e = 0;
    for (int t = 0; t <= trials && e == 0; ++t) {  // trial 0 warms up
      clear_device_flags(c);
      cudaEventRecord(c->stage_ev[0], c->stream);
      bh::launch_walk_variant(c, v, n, (float)theta, (float)eps, scratch, batch);
      cudaEventRecord(c->stage_ev[1], c->stream);
      status = last_launch();
      if (status == BH_OK) status = sync_and_check(c, &e);
      if (status != BH_OK) break;
      if (t > 0) ms.push_back(elapsed(c, 0, 1));
    }
    if (status != BH_OK) break;
    if (e || ms.empty()) {  // this shape cannot run the tree (stack): never chosen
      out->ms[v] = -1.f;
      continue;
    }
    std::sort(ms.begin(), ms.end());
    out->ms[v] = ms[ms.size() / 2];
    if (best_ms == 0.f || out->ms[v] < best_ms) {
      best_ms = out->ms[v];
      best = v;
    }
  }
  dfree(scratch);
  BH_TRY(status);
  if (best_ms == 0.f) return BH_ERR_OVERFLOW_STACK;
  out->variants = nv;
  out->best = best;
  if (c->walk_variant != best) destroy_graphs(c);  // captured batched steps hold the old kernel
  c->walk_variant = best;
  clear_device_flags(c);
  return BH_OK;
}

bh_status bh_set_walk_variant(bh_ctx* c, int variant) {
  if (!c || variant < 0 || variant >= std::min(bh::walk_variants(), (int)BH_TUNE_MAX_VARIANTS))
    return BH_ERR_INVALID_ARG;
  if (c->walk_variant != variant) destroy_graphs(c);
  c->walk_variant = variant;
  return BH_OK;
}

}  // extern "C"
