// Stable LSD radix sort of (u64 key, u32 value) pairs: one histogram pass over all digits,
// then one "onesweep" pass per 8-bit digit (Adinets & Merrill, 2022): each block ranks a
// 4096-key tile with warp-match multisplit, publishes its digit counts, resolves its global
// offsets with a decoupled look-back over the preceding tiles, stages the tile in shared
// memory in digit order and writes every digit run contiguously.
//
// Replaces ThreePassRadixSortMortonKeys / RadixSortPass (src/MortonKeys.hpp:373-470): the
// reference runs stable byte passes at shifts 0,8,16,21,29,37,42,50,58, which together are a
// full stable sort by the 64-bit key; this sort produces the same permutation with passes at
// shifts 0,8,...,56. Stability: within a tile keys are ranked in input order (warp-major,
// then item, then lane, which is the load order), and tiles are ordered by the look-back.
#include <cuda_runtime.h>

#include <mutex>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
#ifndef BH_SORT_ITEMS
#define BH_SORT_ITEMS 16
#endif
#ifndef BH_SORT_MIN_BLOCKS
#define BH_SORT_MIN_BLOCKS 3
#endif
constexpr int kItems = BH_SORT_ITEMS;     // keys per thread
constexpr int kTile = kThreads * kItems;  // 4096 keys
constexpr int kPasses = 8;
constexpr int kRadix = 256;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1;
constexpr int kSpinLimit = 1 << 22;  // about a second of polling; then the sort reports a timeout
constexpr int kLookWindow = 8;       // predecessor tiles read per look-back round trip


__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Digit counts of all 8 passes in one read of the keys. Each thread walks a contiguous run of
// keys and run-length-merges equal digits before touching shared memory: the keys arrive in
// the previous step's sorted order, so the high digits come in long runs.
__global__ __launch_bounds__(kThreads) void k_hist(const uint64_t* __restrict__ keys, int n,
                                                   uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[kPasses * kRadix];
  for (int i = threadIdx.x; i < kPasses * kRadix; i += kThreads) sh[i] = 0;
  __syncthreads();
  constexpr int kRun = 8;
  const long long stride = (long long)gridDim.x * kThreads * kRun;
  for (long long base = ((long long)blockIdx.x * kThreads + threadIdx.x) * kRun; base < n; base += stride) {
    uint32_t cur[kPasses], cnt[kPasses];
#pragma unroll
    for (int p = 0; p < kPasses; ++p) cnt[p] = 0, cur[p] = 0;
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
      long long i = base + j;
      if (i < n) {
        uint64_t k = keys[i];
#pragma unroll
        for (int p = 0; p < kPasses; ++p) {
          uint32_t d = (uint32_t)(k >> (8 * p)) & 0xFFu;
          if (cnt[p] && d != cur[p]) {
            atomicAdd(&sh[p * kRadix + cur[p]], cnt[p]);
            cnt[p] = 0;
          }
          cur[p] = d;
          cnt[p] += 1;
        }
      }
    }
#pragma unroll
    for (int p = 0; p < kPasses; ++p)
      if (cnt[p]) atomicAdd(&sh[p * kRadix + cur[p]], cnt[p]);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kPasses * kRadix; i += kThreads) {
    uint32_t v = sh[i];
    if (v) atomicAdd(&hist[i], v);
  }
}

// Exclusive scan of each pass's 256 digit counts, in place. One block per pass.
__global__ __launch_bounds__(kRadix) void k_hist_scan(uint32_t* __restrict__ hist) {
  __shared__ uint32_t warp_tot[kRadix / 32];
  uint32_t* h = hist + blockIdx.x * kRadix;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  uint32_t v = h[t], x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  uint32_t add = 0;
  for (int i = 0; i < w; ++i) add += warp_tot[i];
  h[t] = x - v + add;
}

struct OnesweepSmem {
  uint64_t keys[kTile];
  uint32_t vals[kTile];
  uint32_t warp_cnt[kWarps][kRadix];
  uint32_t digit_start[kRadix];
  uint32_t global_base[kRadix];
  uint32_t warp_tot[kWarps];
  uint32_t tile;
};

// Three resident blocks per SM (80 registers; the shared-memory tile allows three).
__global__ __launch_bounds__(kThreads, BH_SORT_MIN_BLOCKS) void k_onesweep(const uint64_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin,
                                                       uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                       int n, int shift, const uint32_t* __restrict__ digit_off,
                                                       uint32_t* __restrict__ lookback,
                                                       uint32_t* __restrict__ tile_ctr, uint32_t* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  OnesweepSmem& s = *reinterpret_cast<OnesweepSmem*>(smem_raw);
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;

  if (t == 0) s.tile = atomicAdd(tile_ctr, 1u);
  for (int i = t; i < kWarps * kRadix; i += kThreads) (&s.warp_cnt[0][0])[i] = 0;
  __syncthreads();
  const uint32_t tile = s.tile;
  const long long base = (long long)tile * kTile;
  const int valid_count = (int)min((long long)kTile, (long long)n - base);

  // the keys only: the values are read when the tile is staged, after the ranking, which keeps
  // the ranking at 80 registers and three blocks per SM (two at 128 with the values held from
  // the start: 0.669 -> 0.623 ms per sort at 2^23 keys, 4.62 -> 4.09 ms at 4.7e7)
  uint64_t key[kItems];
  uint32_t rank[kItems];
  const long long wbase = base + (long long)w * (32 * kItems);
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    long long idx = wbase + j * 32 + lane;
    bool ok = idx < n;
    key[j] = ok ? kin[idx] : 0ull;
  }
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    long long idx = wbase + j * 32 + lane;
    bool ok = idx < n;
    uint32_t d = (uint32_t)(key[j] >> shift) & 0xFFu;
    // lanes holding the same digit: one ballot per digit bit (a multisplit by ballots, which
    // issues faster than the match instruction); invalid lanes are nobody's peers
    uint32_t peers = __ballot_sync(0xffffffffu, ok);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const bool bit = (d >> b) & 1u;
      const uint32_t vote = __ballot_sync(0xffffffffu, bit);
      peers &= bit ? vote : ~vote;
    }
    uint32_t pre = ok ? s.warp_cnt[w][d] : 0u;
    __syncwarp();
    if (ok && lane == __ffs(peers) - 1) s.warp_cnt[w][d] = pre + __popc(peers);
    __syncwarp();
    rank[j] = pre + __popc(peers & lt_mask);
  }
  __syncthreads();

  // per-digit: warp-exclusive offsets and the tile total (thread t owns digit t)
  uint32_t total = 0;
#pragma unroll
  for (int ww = 0; ww < kWarps; ++ww) {
    uint32_t c = s.warp_cnt[ww][t];
    s.warp_cnt[ww][t] = total;
    total += c;
  }
  // publish this tile's aggregate (tile 0 publishes its inclusive prefix directly)
  uint32_t* my_lb = lookback + (size_t)tile * kRadix + t;
  st_relaxed(my_lb, (tile == 0 ? kFlagPrefix : kFlagAgg) | total);

  // block-local exclusive scan over digits -> start of each digit run in the staged tile
  uint32_t x = total;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s.warp_tot[w] = x;
  __syncthreads();
  uint32_t add = 0;
  for (int i = 0; i < w; ++i) add += s.warp_tot[i];
  s.digit_start[t] = x - total + add;
  __syncthreads();

  // stage the tile in digit order
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    long long idx = wbase + j * 32 + lane;
    if (idx < n) {
      uint32_t d = (uint32_t)(key[j] >> shift) & 0xFFu;
      uint32_t lp = s.digit_start[d] + s.warp_cnt[w][d] + rank[j];
      s.keys[lp] = key[j];
      s.vals[lp] = vin[idx];
    }
  }

  // decoupled look-back for digit t, reading a window of kLookWindow predecessors per round
  // trip (independent loads in flight together) instead of one tile at a time
  uint32_t excl = 0;
  if (tile > 0) {
    long long k = (long long)tile - 1;
    int spins = 0;
    while (k >= 0) {
      uint32_t v[kLookWindow];
#pragma unroll
      for (int q = 0; q < kLookWindow; ++q)  // tile 0 always holds a prefix, so k - q < 0 is never consumed
        v[q] = (k - q >= 0) ? ld_relaxed(lookback + (size_t)(k - q) * kRadix + t) : kFlagPrefix;
      int used = 0;
      bool done = false;
#pragma unroll
      for (int q = 0; q < kLookWindow; ++q) {
        if (done || used < q) continue;  // stop at a prefix or at the first tile not yet published
        const uint32_t flag = v[q] & ~kValMask;
        if (flag == 0) continue;
        excl += v[q] & kValMask;
        used = q + 1;
        done = flag == kFlagPrefix;
      }
      if (done) break;
      k -= used;
      if (used == 0) {
        if (++spins > kSpinLimit) {
          atomicOr(err, kErrTimeout);
          break;
        }
        __nanosleep(32);
      }
    }
    st_relaxed(my_lb, kFlagPrefix | ((excl + total) & kValMask));
  }
  s.global_base[t] = digit_off[t] + excl;
  __syncthreads();

  for (int i = t; i < valid_count; i += kThreads) {
    uint64_t kk = s.keys[i];
    uint32_t d = (uint32_t)(kk >> shift) & 0xFFu;
    uint32_t gp = s.global_base[d] + (uint32_t)i - s.digit_start[d];
    if (gp < (uint32_t)n) {  // always true unless a look-back wait timed out (flagged above)
      kout[gp] = kk;
      vout[gp] = s.vals[i];
    }
  }
}

// ---------------------------------------------------------------------------------------
// Small sorts by rank counting. Each key's output position is the number of keys that sort
// before it: the smaller keys, and the equal keys earlier in the input (which makes the sort
// stable). A block takes 32 consecutive keys i, one per lane, and its eight warps split each
// staged tile of keys j into eighths; all lanes of a warp compare their key with the same j (a
// shared-memory broadcast), and the block adds the eight partial counts. That is n^2
// comparisons spread over the whole GPU (about 20 M at 4 444 keys), where the eight digit passes
// of a radix sort are a chain of launches, or of barriers inside one block, that costs far more
// at this size.
// ---------------------------------------------------------------------------------------
constexpr int kRankThreads = 256;
constexpr int kRankParts = kRankThreads / 32;
#ifndef BH_RANK_TILE
#define BH_RANK_TILE 4096
#endif
// keys j staged per round (8 bytes each): 2048 / 4096 / 5120 give 67.0 / 63.6 / 69.4 us per sort
// at 16 384 keys and 16.6 / 16.4 / 14.4 us at 4 444
constexpr int kRankTile = BH_RANK_TILE;
// Sorts of at most this many keys go by rank: at 4 444 keys 16 us against the radix sort's
// 68 us, at 16 384 keys 66 us against 74 us (the n^2 comparisons catch up beyond).
constexpr int kRankSortMax = 16384;

__global__ __launch_bounds__(kThreads) void k_copy_pairs(const uint64_t* __restrict__ kin,
                                                         const uint32_t* __restrict__ vin,
                                                         uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                         int n) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < n) {
    kout[i] = kin[i];
    vout[i] = vin[i];
  }
}

__global__ __launch_bounds__(kRankThreads) void k_sort_rank(const uint64_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                            int n) {
  __shared__ uint64_t s_k[kRankTile];
  __shared__ uint32_t s_cnt[kRankParts][32];
  const int lane = threadIdx.x & 31, part = threadIdx.x >> 5;
  const int base = blockIdx.x * 32, i = base + lane;
  const bool valid = i < n;
  const uint64_t ki = valid ? kin[i] : 0ull;
  uint32_t cnt = 0;
  // the keys j come through shared memory a tile at a time (one coalesced read of the tile by the
  // block, instead of a chain of dependent-latency broadcast reads from L2 per warp); warp `part`
  // compares its lanes' keys with its eighth of the tile
  for (int t0 = 0; t0 < n; t0 += kRankTile) {
    const int m = min(kRankTile, n - t0);
#pragma unroll
    for (int r = 0; r < kRankTile / kRankThreads; ++r) {
      const int q = r * kRankThreads + threadIdx.x;
      if (q < m) s_k[q] = kin[t0 + q];
    }
    __syncthreads();
    const int j0 = t0 + part * (kRankTile / kRankParts);
    const int j1 = min(t0 + m, j0 + kRankTile / kRankParts);
    const uint64_t* sk = s_k - t0;  // sk[j] is key j
    const int below = min(j1, base);  // j before all of this warp's keys: equal keys sort first
#pragma unroll 8
    for (int j = j0; j < below; ++j) cnt += sk[j] <= ki ? 1u : 0u;
    const int d1 = min(j1, base + 32);  // this warp's own keys: equal ones sort first when j < i
    for (int j = max(j0, base); j < d1; ++j) {
      const uint64_t kj = sk[j];
      cnt += (kj < ki || (kj == ki && j < i)) ? 1u : 0u;
    }
#pragma unroll 8
    for (int j = max(j0, base + 32); j < j1; ++j) cnt += sk[j] < ki ? 1u : 0u;  // after: equal keys sort later
    __syncthreads();
  }
  s_cnt[part][lane] = cnt;
  __syncthreads();
  if (part == 0 && valid) {
    uint32_t r = 0;
#pragma unroll
    for (int q = 0; q < kRankParts; ++q) r += s_cnt[q][lane];
    kout[r] = ki;
    vout[r] = vin[i];
  }
}

}  // namespace

int sort_max_tiles(size_t n) { return (int)((n + kTile - 1) / kTile); }

// Function attributes set once per process, before any stream capture.
void sort_init() {
  cudaFuncSetAttribute(k_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(OnesweepSmem));
}

// Sorts (keys_in, vals_in) stably by the full 64-bit key. The result lands in keys_in /
// vals_in (an even number of passes); the *_tmp buffers are scratch of the same size.
void radix_sort_pairs(bh_ctx* c, uint64_t* keys_in, uint32_t* vals_in, uint64_t* keys_tmp, uint32_t* vals_tmp,
                      int n, cudaStream_t st, uint64_t** keys_out, uint32_t** vals_out, int first_pass,
                      int npasses) {
  *keys_out = keys_in;
  *vals_out = vals_in;
  if (n <= 1) return;
  if (n <= kRankSortMax && first_pass == 0 && npasses == kPasses) {
    // the result goes back to keys_in / vals_in, as after the eight digit passes
    c->launches += 2;
    k_copy_pairs<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(keys_in, vals_in, keys_tmp, vals_tmp, n);
    k_sort_rank<<<(n + 31) / 32, kRankThreads, 0, st>>>(keys_tmp, vals_tmp, keys_in, vals_in, n);
    return;
  }
  const int tiles = sort_max_tiles((size_t)n);
  cudaMemsetAsync(c->sort.hist, 0, sizeof(uint32_t) * kPasses * kRadix, st);
  cudaMemsetAsync(c->sort.lookback, 0, sizeof(uint32_t) * (size_t)kPasses * tiles * kRadix, st);
  cudaMemsetAsync(c->sort.tile_ctr, 0, sizeof(uint32_t) * kPasses, st);
  int hblocks = (int)min((long long)c->sms * 4, ((long long)n + kThreads * 8 - 1) / (kThreads * 8));
  c->launches += 2 + npasses;
  k_hist<<<hblocks, kThreads, 0, st>>>(keys_in, n, c->sort.hist);
  k_hist_scan<<<kPasses, kRadix, 0, st>>>(c->sort.hist);
  uint64_t* ka = keys_in;
  uint32_t* va = vals_in;
  uint64_t* kb = keys_tmp;
  uint32_t* vb = vals_tmp;
  for (int p = first_pass; p < first_pass + npasses; ++p) {
    k_onesweep<<<tiles, kThreads, sizeof(OnesweepSmem), st>>>(ka, va, kb, vb, n, 8 * p, c->sort.hist + p * kRadix,
                                                              c->sort.lookback + (size_t)p * tiles * kRadix,
                                                              c->sort.tile_ctr + p, c->err);
    uint64_t* tk = ka;
    ka = kb;
    kb = tk;
    uint32_t* tv = va;
    va = vb;
    vb = tv;
  }
  *keys_out = ka;
  *vals_out = va;
}

}  // namespace bh

// ---------------------------------------------------------------------------------------
// Allocation-free sort entry point (bh_sort_keys_static, include/bhgpu.h).
//
// Some callers cannot call cudaMalloc at the point where they need a sort: code running in
// a per-frame loop or a chain of stream callbacks, where cudaMalloc / cudaFree would
// synchronise the whole device and stall other streams, and embedders that reserve a fixed
// device-memory budget up front and forbid allocations afterwards. For them this variant keeps
// every scratch buffer the sort needs (ping-pong key/value buffers, digit histograms, look-back
// words, tile counters, error word) in one file-scope __device__ array of fixed size, which
// the GPU holds for as long as the library is loaded. The caller passes only its inputs and
// outputs.
//
// The array's name in host code is only a host-side stand-in for the symbol, not a device
// address; the device address is resolved with cudaGetSymbolAddress the first time the entry
// point runs on a device (with that device current) and cached per device. That first call
// therefore has to happen outside any stream capture. All calls share the one array and each
// call overwrites it, so calls that could overlap on the GPU (different streams without
// ordering, or different host threads) race and must be serialised by the caller.
// ---------------------------------------------------------------------------------------
namespace bh {
namespace {

constexpr size_t kStaticMaxKeys = BH_SORT_STATIC_MAX_KEYS;
constexpr int kStaticTiles = (int)((kStaticMaxKeys + kTile - 1) / kTile);
constexpr size_t kOffTmpKeys = 0;
constexpr size_t kOffTmpVals = kOffTmpKeys + kStaticMaxKeys * sizeof(uint64_t);
constexpr size_t kOffHist = kOffTmpVals + kStaticMaxKeys * sizeof(uint32_t);
constexpr size_t kOffLookback = kOffHist + (size_t)kPasses * kRadix * sizeof(uint32_t);
constexpr size_t kOffTileCtr = kOffLookback + (size_t)kPasses * kStaticTiles * kRadix * sizeof(uint32_t);
constexpr size_t kOffErr = kOffTileCtr + kPasses * sizeof(uint32_t);
constexpr size_t kStaticBytes = kOffErr + 256;

static __device__ __align__(256) unsigned char g_static_sort_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
unsigned char* g_static_addr[kMaxDevices] = {};
bool g_static_attr[kMaxDevices] = {};
int g_static_sms[kMaxDevices] = {};

}  // namespace
}  // namespace bh

extern "C" bh_status bh_sort_keys_static(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                                         uint32_t* vals_out, size_t n, void* stream, uint32_t* status_out) {
  using namespace bh;
  if (n > kStaticMaxKeys) return BH_ERR_INVALID_ARG;
  if (n > 0 && (!keys_in || !vals_in || !keys_out || !vals_out)) return BH_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return BH_ERR_DEVICE;
  }
  unsigned char* base = nullptr;
  int sms = 0;
  {
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_static_sort_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return BH_ERR_DEVICE;
      }
      g_static_addr[dev] = (unsigned char*)p;
    }
    if (!g_static_attr[dev]) {
      if (cudaFuncSetAttribute(k_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)sizeof(OnesweepSmem)) != cudaSuccess) {
        cudaGetLastError();
        return BH_ERR_DEVICE;
      }
      g_static_attr[dev] = true;
    }
    if (!g_static_sms[dev]) {
      if (cudaDeviceGetAttribute(&g_static_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          g_static_sms[dev] <= 0) {
        g_static_sms[dev] = 0;
        cudaGetLastError();
        return BH_ERR_DEVICE;
      }
    }
    base = g_static_addr[dev];
    sms = g_static_sms[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int nn = (int)n;
  if (nn <= 1 && status_out) cudaMemsetAsync(status_out, 0, sizeof(uint32_t), st);
  if (nn == 0) return cudaGetLastError() == cudaSuccess ? BH_OK : BH_ERR_DEVICE;
  if (nn == 1) {
    cudaMemcpyAsync(keys_out, keys_in, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(vals_out, vals_in, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    return cudaGetLastError() == cudaSuccess ? BH_OK : BH_ERR_DEVICE;
  }
  uint64_t* tmp_keys = (uint64_t*)(base + kOffTmpKeys);
  uint32_t* tmp_vals = (uint32_t*)(base + kOffTmpVals);
  uint32_t* hist = (uint32_t*)(base + kOffHist);
  uint32_t* lookback = (uint32_t*)(base + kOffLookback);
  uint32_t* tile_ctr = (uint32_t*)(base + kOffTileCtr);
  uint32_t* err = status_out ? status_out : (uint32_t*)(base + kOffErr);
  const int tiles = sort_max_tiles(n);
  // everything that must start at zero: histograms, look-back words, tile counters, error word
  cudaMemsetAsync(hist, 0, kOffErr + sizeof(uint32_t) - kOffHist, st);
  if (status_out) cudaMemsetAsync(status_out, 0, sizeof(uint32_t), st);
  const int hblocks = (int)min((long long)sms * 4, ((long long)nn + kThreads * 8 - 1) / (kThreads * 8));
  k_hist<<<hblocks, kThreads, 0, st>>>(keys_in, nn, hist);
  k_hist_scan<<<kPasses, kRadix, 0, st>>>(hist);
  // pass p reads from (p == 0 ? input : buffer of pass p - 1) and writes the tmp buffers on
  // even passes and the caller's output on odd ones; 8 passes end in the output
  const uint64_t* ka = keys_in;
  const uint32_t* va = vals_in;
  for (int p = 0; p < kPasses; ++p) {
    uint64_t* kb = (p & 1) ? keys_out : tmp_keys;
    uint32_t* vb = (p & 1) ? vals_out : tmp_vals;
    k_onesweep<<<tiles, kThreads, sizeof(OnesweepSmem), st>>>(ka, va, kb, vb, nn, 8 * p, hist + p * kRadix,
                                                              lookback + (size_t)p * tiles * kRadix,
                                                              tile_ctr + p, err);
    ka = kb;
    va = vb;
  }
  return cudaGetLastError() == cudaSuccess ? BH_OK : BH_ERR_DEVICE;
}
