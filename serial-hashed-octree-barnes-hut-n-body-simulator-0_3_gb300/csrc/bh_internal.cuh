// Internal declarations shared by the libbhgpu translation units (not part of the ABI).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "bhgpu.h"

namespace bh {

// NVTX range over a host scope: names each library call in profiler timelines (header-only
// NVTX 3; without an attached tool a push/pop is a no-op call).
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};

constexpr int kMaxDepth = 21;             // 21 bits per axis, 63-bit keys (reference: MortonKeys.hpp:42)
constexpr int kLevels = kMaxDepth + 1;    // depths 0..21
constexpr int kNumEvents = 64;
// Levels with at most this many nodes are built one warp per node (tiles of 8 nodes): one
// resident wave of the build's 608 blocks x 8 warps.
constexpr int kLevelWarpNodes = 4864;

// Device error word bits. bit = (bh_status code - 3), so the host maps them back.
enum : uint32_t {
  kErrStack = 1u << (BH_ERR_OVERFLOW_STACK - 3),
  kErrHash = 1u << (BH_ERR_OVERFLOW_HASH - 3),
  kErrNodes = 1u << (BH_ERR_OVERFLOW_NODES - 3),
  kErrTimeout = 1u << (BH_ERR_TIMEOUT - 3),
  kErrTape = 1u << (BH_ERR_OVERFLOW_TAPE - 3),
};

// Geometry of one step, produced on the device by the bounds kernel (or set by the host
// for caller-given bounds) and read by the key kernels.
struct Geom {
  double center[3];  // OctantBounds::center
  double size;       // OctantBounds::size (S)
  double frac;       // 2^21 / (2 S): Morton scale
  double tc[3];      // tree root centre
  double tedge;      // tree root edge
  double tscale;     // 2^21 / tedge
  double tmargin;    // fast-path margin in key units (see tree_key)
  // float-float splits (value = hi + lo) of the fields above for the FP32 fast paths of the
  // key kernels (GB300's FP64 pipe is far slower than its FP32 pipe)
  float size_hi, size_lo, frac_hi, frac_lo;
  float tc_hi[3], tc_lo[3];
  float tscale_hi, tscale_lo, tmargin_f;
};

// Walk record of one node: 64 bytes, read by the tree walk.
//   mac : centre of mass (x, y, z) and edge^2; edge^2 is stored negated for single-body
//         leaves so the walk can route them to the point list without another load.
//   mq  : mass, Qxx, Qxy, Qxz
//   q2  : Qyy, Qyz, Qzz, unused
//   link: first child, child count, first body (tree order), body count
struct __align__(16) WalkNode {
  float4 mac;
  float4 mq;
  float4 q2;
  int4 link;
};

// Multipole of one node, kept for the parents during the upsweep (64 bytes). Mass and
// centre of mass are float-float pairs (value = hi + lo, about 44 significant bits, from
// compensated FP32 sums: GB300's FP64 pipe is far too slow for this pass); the quadrupole is
// FP32. hi is the FP32 rounding of the pair, which is what the walk reads.
struct __align__(16) NodeUp {
  float com_hi[3];
  float mass_hi;
  float com_lo[3];
  float mass_lo;
  float q[6];         // Qxx, Qxy, Qxz, Qyy, Qyz, Qzz about the centre of mass
  uint32_t min_rank;  // smallest Morton slot among members (literal barycentre)
  uint32_t pad;
};

// One recorded evaluation buffer of the walk (the adjoint replays these): the group it served
// (first body in tree order, body count), the kind (0 cells, 1 points), the entry count, and
// per entry the node (cells) or point index (>= 0 body in tree order, < 0 -(node + 1)) and the
// 32-bit mask of lanes that took it.
struct __align__(16) Chunk {
  int4 hdr;
  int idx[32];
  uint32_t mask[32];
};

struct Counters {
  unsigned long long cell;
  unsigned long long p2p;
  unsigned long long cell_evals;   // warp-wide cell entries evaluated (32 lane slots each)
  unsigned long long point_evals;  // warp-wide point entries evaluated
  unsigned int group_next;  // walk work queue
  unsigned int max_depth;
};

// Radix sort (onesweep) scratch.
struct SortScratch {
  uint32_t* hist = nullptr;        // [8][256] digit counts, then exclusive offsets
  uint32_t* lookback = nullptr;    // [8][max_tiles][256]
  uint32_t* tile_ctr = nullptr;    // [8]
  int max_tiles = 0;
};

struct Arena {
  void* base = nullptr;
  size_t bytes = 0;
};

}  // namespace bh

struct bh_ctx {
  int device = 0;
  int sms = 0;  // streaming multiprocessors of the device (grid sizing)
  size_t cap = 0;  // bodies
  size_t n = 0;
  cudaStream_t stream = nullptr;      // where the context's work runs (own_stream or the caller's)
  cudaStream_t own_stream = nullptr;  // created with the context; every graph capture runs on it
  cudaEvent_t ev[bh::kNumEvents] = {};
  cudaEvent_t stage_ev[16] = {};

  // body state (Morton order), ping-pong
  float4* pos[2] = {nullptr, nullptr};
  float4* vel[2] = {nullptr, nullptr};
  float4* acc = nullptr;
  int cur = 0;

  // keys / sort
  uint64_t* keys[2] = {nullptr, nullptr};
  uint32_t* vals[2] = {nullptr, nullptr};
  uint64_t* body_key = nullptr;  // last Morton keys, per slot
  bh::SortScratch sort;

  // tree (over the bodies in tree-key order)
  uint64_t* tkey = nullptr;   // sorted tree keys
  uint32_t* tslot = nullptr;  // tree order -> body slot
  float4* tpos = nullptr;     // positions+mass in tree order
  size_t node_cap = 0;
  uint64_t* nkey = nullptr;
  int2* nrange = nullptr;  // first body, body count
  bh::WalkNode* wnode = nullptr;
  bh::NodeUp* nup = nullptr;
  uint8_t* nchildbyte = nullptr;
  int* nparent = nullptr;      // parent node (-1 for roots), for the upsweep
  uint32_t* narrived = nullptr;  // upsweep: children finished, per node
  uint32_t* lb_level = nullptr;  // look-back words of the level build
  int lb_level_tiles = 0;
  int* level_bounds = nullptr;  // [kLevels + 1] node index where each depth starts
  uint32_t* level_tile_ctr = nullptr;  // [kLevels]
  uint64_t* hash_keys = nullptr;
  int* hash_vals = nullptr;
  size_t hash_cap = 0;
  bool hash_valid = false;
  bool tree_valid = false;
  int tree_leaf_cap = 1;
  int tree_mode = 1;
  double tree_center[3] = {0, 0, 0};
  double tree_edge = 0;

  bh::Geom* geom = nullptr;  // device
  double* bounds_partial = nullptr;
  int bounds_blocks = 0;
  uint32_t* err = nullptr;
  bh::Counters* counters = nullptr;

  // host mirror of small device results
  uint32_t* h_err = nullptr;  // pinned
  bh::Counters* h_counters = nullptr;
  int* h_level_bounds = nullptr;

  void* flush_buf = nullptr;
  size_t flush_bytes = 0;

  // batched ensemble (bh_batch_*): system s owns the fixed body range [sys_off[s], sys_off[s+1])
  bool batch = false;
  int nsys = 0;
  uint32_t* sys_off = nullptr;     // device [nsys + 1]
  uint16_t* body_sys = nullptr;    // device, system of each body slot / tree position
  bh::Geom* sys_geom = nullptr;    // device [nsys]
  int4* groups = nullptr;          // device walk groups: first body, body count, root node, system
  int ngroups = 0;
  size_t sys_cap = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // captured batched step, by state parity
  bh_params graph_params = {};
  uint64_t graph_kernels[2] = {0, 0};  // kernel launches inside each captured graph
  uint64_t* graph_keys0[2] = {nullptr, nullptr};  // plain step graphs: the key buffer they were captured with
  // whether each graph records the per-stage events (captured so only for calls that return
  // stats: each event-record node costs about 4.6 us of graph time)
  bool graph_marks[2] = {false, false};
  bool host_graph_marks[2] = {false, false};
  size_t graph_n = 0;                              // plain step graphs: the body count they were captured for
  // bh_step_host: the step with its host copies on a second stream, one graph per state parity
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t io_ev[4] = {};  // fork, velocities uploaded, positions final, positions downloaded
  cudaGraphExec_t host_graph[2] = {nullptr, nullptr};
  const void* host_graph_ptrs[2][4] = {};  // the host buffers each was captured with
  uint64_t* host_graph_keys0[2] = {nullptr, nullptr};
  uint64_t host_graph_kernels[2] = {0, 0};
  uint64_t launches = 0;  // kernels launched on this context (every launcher adds its count)

  void* adj = nullptr;  // differentiable-path state (checkpoints, tape, adjoints): bh_adjoint.cu

  int walk_variant = 0;           // launch shape of the quadrupole walk (bh_autotune_walk)
  bool batch_tree_ready = false;  // the arena holds the tree of the last batched step
};

namespace bh {

// ---- host helpers (bh_api.cu) ----
template <class T>
inline bh_status dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (cudaMalloc((void**)p, sizeof(T) * count) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return BH_ERR_OOM;
  }
  return BH_OK;
}

template <class T>
inline void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

#define BH_TRY(expr)            \
  do {                          \
    bh_status s_ = (expr);      \
    if (s_ != BH_OK) return s_; \
  } while (0)

bh_status cuda_status(cudaError_t e);
bh_status last_launch();
bh_status err_to_status(uint32_t e);
bh_status ensure_nodes(bh_ctx* c, size_t need);
// Reads the device error word, the counters and the level bounds after finishing the stream.
bh_status sync_and_check(bh_ctx* c, uint32_t* err_out = nullptr);
void clear_device_flags(bh_ctx* c);
float elapsed(bh_ctx* c, int a, int b);

// Kernel launchers (defined in the .cu files; all asynchronous on `st`).
// Stable LSD radix sort by 8-bit digits first_pass .. first_pass + npasses - 1 of the keys
// (all 8 digits by default). With an even pass count the result is back in keys_in / vals_in.
void radix_sort_pairs(bh_ctx* c, uint64_t* keys_in, uint32_t* vals_in, uint64_t* keys_tmp, uint32_t* vals_tmp,
                      int n, cudaStream_t st, uint64_t** keys_out, uint32_t** vals_out, int first_pass = 0,
                      int npasses = 8);
int sort_max_tiles(size_t n);
void sort_init();
void walk_init();
void tree_init();

void launch_bounds(bh_ctx* c, const float4* pos, int n, double edge_factor);
void launch_set_geom(bh_ctx* c, const double center[3], double size, const double tcenter[3], double tedge);
void launch_morton(bh_ctx* c, const float4* pos, int n, uint64_t* keys, uint32_t* idx, bool batch = false);
void launch_decode_morton(bh_ctx* c, const uint64_t* keys, int n, double size, double* pos3);
void launch_gather(bh_ctx* c, const uint32_t* perm, int n, const float4* pin, const float4* vin, float4* pout,
                   float4* vout);
void launch_gather_kd_treekey(bh_ctx* c, const uint32_t* perm, int n, const float4* pin, const float4* vin,
                              const float4* acc, int acc_follows_body, float dt, float4* pout, float4* vout,
                              uint64_t* tkeys, uint32_t* tidx, bool batch = false);
void launch_treekey(bh_ctx* c, const float4* pos, int n, uint64_t* tkeys, uint32_t* tidx);
void launch_kick_drift(bh_ctx* c, float4* pos, float4* vel, const float4* acc, int n, float dt, int drift);
void launch_gather_tree(bh_ctx* c, const uint32_t* tslot, int n, const float4* pos, float4* tpos);
void launch_build(bh_ctx* c, int n, int leaf_cap, bool batch = false);
void launch_upsweep(bh_ctx* c, int n, int leaf_cap, int mode, bool batch = false);
void launch_batch_bounds(bh_ctx* c, const float4* pos, double edge_factor);
void launch_sys_keys(bh_ctx* c, const uint32_t* vals, int n, uint64_t* k2);
void launch_gather_tree_keys(bh_ctx* c, const uint32_t* tslot, int n, const float4* pos,
                             const uint64_t* key_by_slot, float4* tpos, uint64_t* tkey);
void launch_hash(bh_ctx* c);
// vel_copy (optional, with vel_kick): a second destination of the kicked velocities, such as a
// caller's mapped pinned host buffer
void launch_walk(bh_ctx* c, int n, float theta, float eps, int mode, float4* acc_slot, float4* vel_kick,
                 float half_dt, bool batch = false, float4* vel_copy = nullptr);
void launch_lookup(bh_ctx* c, uint64_t key, int* out_index);
void launch_walk_record(bh_ctx* c, int n, float theta, float eps, float4* acc_slot, float4* vel_kick, float half_dt,
                        Chunk* tape, unsigned* tape_count, int tape_cap);
void launch_fp32_peak(cudaStream_t st, float* sink, int blocks);
// Launch shapes of the quadrupole walk (positive softening) that bh_autotune_walk times.
struct WalkVariant {
  int warps, min_blocks, stack, form, regs, group;  // group: bodies per warp (single systems)
};
int walk_variants();
WalkVariant walk_variant_info(int v);
void launch_walk_variant(bh_ctx* c, int v, int n, float theta, float eps, float4* acc_out, bool batch);

// Frees the differentiable-path state of the context.
void adj_release(bh_ctx* c);
// Marks the recorded trajectory stale (new bodies were uploaded).
void adj_invalidate(bh_ctx* c);
// New state of n bodies (bh_api.cu): derived structures dropped, accelerations and keys zeroed.
void reset_state(bh_ctx* c, size_t n);
// Ensemble layout over the bodies already in the state (bh_api.cu).
bh_status check_sys_offsets(const bh_ctx* c, const uint32_t* sys_offsets, size_t nsys);
bh_status batch_layout(bh_ctx* c, const uint32_t* sys_offsets, size_t nsys);

}  // namespace bh
