// Device-wide exclusive scan and stable LSD radix sort (sm_103a), plus the C-ABI error
// plumbing.  The scan is one pass with decoupled look-back: a block waits only for tiles
// whose blocks are already running, and every wait is bounded.  The radix sort is
// reduce-then-scan: its blocks never wait on one another.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "sph_common.cuh"

namespace sph {

static thread_local char g_err[512] = "";

void set_error(const char* where, cudaError_t err) {
  snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(err));
}
void set_error_text(const char* text) { snprintf(g_err, sizeof(g_err), "%s", text); }

// ------------------------------------------------------------------ scan
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096

// Shared-memory index of tile item i, one pad word per 32: a thread's kScanItems
// consecutive items (i = kScanItems * t + k) and a warp's coalesced column (i = 256 k + t)
// then both fall in 32 distinct banks.
__device__ __forceinline__ int tpad(int i) { return i + (i >> 5); }
constexpr int kScanTilePadded = kScanTile + kScanTile / 32;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total via *total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* smem_warp, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  T incl = warp_incl_scan(v);
  if (lane == 31) smem_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nwarps ? smem_warp[lane] : T(0);
    T wi = warp_incl_scan(w);
    if (lane < nwarps) smem_warp[lane] = wi - w;
    if (lane == nwarps - 1) smem_warp[32] = wi;
  }
  __syncthreads();
  T res = incl - v + smem_warp[warp];
  *total = smem_warp[32];
  __syncthreads();
  return res;
}

// Small scans in one launch: one block walks the tiles in order with a running carry
// (n <= kSmallScanItems; the look-back scan needs its tile words zeroed first, one more
// operation in a small scene's step).
constexpr int64_t kSmallScanItems = 4 * (int64_t)kScanTile;

template <typename TOut>
__global__ void __launch_bounds__(kScanThreads) k_scan_small(const int32_t* __restrict__ in, TOut* __restrict__ out,
                                                             int64_t n) {
  __shared__ TOut sw[33];
  __shared__ TOut tile[kScanTilePadded];
  TOut carry = 0;
  for (int64_t base = 0; base < n; base += kScanTile) {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      const int64_t idx = base + (int64_t)k * kScanThreads + threadIdx.x;
      tile[tpad(k * kScanThreads + threadIdx.x)] = idx < n ? (TOut)in[idx] : TOut(0);
    }
    __syncthreads();
    TOut local[kScanItems];
    TOut sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      local[k] = sum;
      sum += tile[tpad(threadIdx.x * kScanItems + k)];
    }
    TOut total;
    const TOut ex = block_excl_scan<TOut>(sum, sw, &total) + carry;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) tile[tpad(threadIdx.x * kScanItems + k)] = ex + local[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      const int64_t idx = base + (int64_t)k * kScanThreads + threadIdx.x;
      if (idx < n) out[idx] = tile[tpad(k * kScanThreads + threadIdx.x)];
    }
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

static int64_t scan_blocks(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

// Single-pass scan by decoupled look-back (Merrill and Garland, "Single-pass Parallel Prefix
// Scan with Decoupled Look-back", 2016).  A block takes the next tile by ticket, publishes
// the tile's total, then warp 0 walks back over the tiles before it 32 at a time, adding
// their totals until it meets a published inclusive prefix, and publishes its own.  Tile
// words pack a 2-bit state (0 not ready, 1 total, 2 inclusive prefix) over a 62-bit
// two's-complement value, so state and value are stored and loaded as one 64-bit word.
// Tile t waits only for tiles with smaller tickets: their blocks are resident and publish
// their totals before they wait on anything, so each wait ends.  Each poll loop is still
// bounded (kLookbackPolls); a block that gives up counts a timeout in g_scan_timeouts
// (read by sph_scan_timeouts) and leaves its output wrong rather than spin on.
constexpr unsigned long long kTileTotal = 1ull << 62, kTilePrefix = 2ull << 62;
constexpr unsigned long long kTileValue = (1ull << 62) - 1;
constexpr int kLookbackPolls = 1 << 20;
static __device__ unsigned long long g_scan_timeouts;

__device__ __forceinline__ void tile_publish(unsigned long long* w, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(w), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long tile_peek(const unsigned long long* w) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(w) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long tile_word(unsigned long long state, int64_t v) {
  return state | ((unsigned long long)v & kTileValue);
}

__device__ __forceinline__ int64_t tile_value(unsigned long long w) { return (int64_t)(w << 2) >> 2; }

// tiles: ntiles zeroed words and the ticket counter after them (zeroed).
template <typename TOut>
__global__ void __launch_bounds__(kScanThreads) k_scan_lookback(const int32_t* __restrict__ in, TOut* __restrict__ out,
                                                                int64_t n, unsigned long long* tiles,
                                                                int64_t ntiles) {
  __shared__ TOut sw[33];
  __shared__ TOut tile[kScanTilePadded];
  __shared__ int64_t s_t;
  __shared__ TOut s_prefix;
  if (threadIdx.x == 0) s_t = (int64_t)atomicAdd(tiles + ntiles, 1ull);
  __syncthreads();
  const int64_t t = s_t;
  const int64_t base = t * kScanTile;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t idx = base + (int64_t)k * kScanThreads + threadIdx.x;
    tile[tpad(k * kScanThreads + threadIdx.x)] = idx < n ? (TOut)in[idx] : TOut(0);
  }
  __syncthreads();
  TOut local[kScanItems];
  TOut sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    local[k] = sum;
    sum += tile[tpad(threadIdx.x * kScanItems + k)];
  }
  TOut total;
  const TOut ex = block_excl_scan<TOut>(sum, sw, &total);
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (lane == 0) tile_publish(tiles + t, tile_word(t == 0 ? kTilePrefix : kTileTotal, (int64_t)total));
    TOut excl = 0;
    if (t > 0) {
      int64_t j = t - 1;   // the nearest tile of this window
      int polls = 0;
      while (true) {
        const int64_t k = j - lane;
        const unsigned long long w = k >= 0 ? tile_peek(tiles + k) : kTilePrefix;
        const unsigned long long state = w & ~kTileValue;
        const unsigned pre = __ballot_sync(0xffffffffu, state == kTilePrefix);
        const unsigned pending = __ballot_sync(0xffffffffu, state == 0);
        const unsigned upto = pre ? ((pre & (0u - pre)) << 1) - 1u : 0xffffffffu;   // lanes up to the first prefix
        if (pending & upto) {
          if (++polls > kLookbackPolls) {
            if (lane == 0) atomicAdd(&g_scan_timeouts, 1ull);
            break;
          }
          __nanosleep(64);
          continue;
        }
        TOut v = ((upto >> lane) & 1u) ? (TOut)tile_value(w) : TOut(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        excl += v;
        if (pre) break;
        j -= 32;
      }
      if (lane == 0) tile_publish(tiles + t, tile_word(kTilePrefix, (int64_t)(excl + total)));
    }
    if (lane == 0) s_prefix = excl;
  }
  __syncthreads();
  const TOut off = ex + s_prefix;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) tile[tpad(threadIdx.x * kScanItems + k)] = off + local[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t idx = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (idx < n) out[idx] = tile[tpad(k * kScanThreads + threadIdx.x)];
  }
  if (t == ntiles - 1 && threadIdx.x == 0) out[n] = s_prefix + total;
}

template <typename TOut>
static sph_status_t scan_impl(const int32_t* in, TOut* out, int64_t n, void* scratch, size_t scratch_bytes,
                              void* stream) {
  SPH_REQUIRE(n >= 0 && out != nullptr, "scan: bad arguments");
  cudaStream_t st = as_stream(stream);
  if (n == 0) {
    cudaMemsetAsync(out, 0, sizeof(TOut), st);
    SPH_CHECK_LAUNCH("scan(memset)");
    return SPH_OK;
  }
  int64_t nb = scan_blocks(n);
  // the tile words are 64-bit atomics: start them on an 8-byte boundary
  const size_t skip = scratch ? (size_t)((8 - (reinterpret_cast<uintptr_t>(scratch) & 7)) & 7) : 0;
  if (scratch == nullptr || scratch_bytes < skip + (size_t)(nb + 1) * sizeof(int64_t)) {
    set_error_text("scan: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  scratch = static_cast<char*>(scratch) + skip;
  if (n <= kSmallScanItems) {
    k_scan_small<TOut><<<1, kScanThreads, 0, st>>>(in, out, n);
    SPH_CHECK_LAUNCH("scan(small)");
    return SPH_OK;
  }
  unsigned long long* tiles = reinterpret_cast<unsigned long long*>(scratch);
  cudaMemsetAsync(tiles, 0, (size_t)(nb + 1) * sizeof(unsigned long long), st);
  k_scan_lookback<TOut><<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, tiles, nb);
  SPH_CHECK_LAUNCH("scan");
  return SPH_OK;
}

// ------------------------------------------------------------------ allocation-free scan
// Scratch for sph_exclusive_scan_i32_static: one 64-bit tile word per 4096-item tile plus
// the ticket counter.  64 KiB of device memory in every GPU that loads this library, held until
// the process exits.  It caps n at (kStaticScanSlots - 1) * kScanTile = 33,550,336 items.
constexpr int kStaticScanSlots = 8192;
static __device__ __align__(256) int64_t g_static_scan_scratch[kStaticScanSlots];

constexpr int kMaxDevices = 64;
static void* g_static_scan_ptr[kMaxDevices] = {nullptr};
static std::mutex g_static_scan_mu;

// Device address of g_static_scan_scratch for the current device.  The host-side symbol
// is only a stand-in: kernels must be given this address.  Looked up once per device.
static sph_status_t static_scan_scratch(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("static scan: cudaGetDevice", e);
    return SPH_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error_text("static scan: device index out of range");
    return SPH_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_static_scan_mu);
  if (g_static_scan_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scan_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error("static scan: cudaGetSymbolAddress", e);
      return SPH_ERR_CUDA;
    }
    g_static_scan_ptr[dev] = p;
  }
  *out = g_static_scan_ptr[dev];
  return SPH_OK;
}

// ------------------------------------------------------------------ radix sort
constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsRounds = 8;
constexpr int kRsTile = kRsThreads * kRsRounds;  // 2048 keys per block

__global__ void __launch_bounds__(kRsThreads) k_radix_hist(const uint32_t* __restrict__ keys, int64_t n, int shift,
                                                           int digit_bits, int32_t* __restrict__ hist, int ntiles) {
  __shared__ int32_t cnt[256];
  const int nd = 1 << digit_bits;
  const uint32_t mask = (uint32_t)nd - 1u;
  for (int d = threadIdx.x; d < nd; d += kRsThreads) cnt[d] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    int64_t idx = base + (int64_t)r * kRsThreads + threadIdx.x;
    if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & mask], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nd; d += kRsThreads) hist[(int64_t)d * ntiles + blockIdx.x] = cnt[d];
}

// Stable scatter: tile order = (round, warp, lane); the rank of an item among equal
// digits is (count in earlier rounds) + (count in earlier warps of this round) +
// (count among earlier lanes, from __match_any_sync).
__global__ void __launch_bounds__(kRsThreads) k_radix_scatter(const uint32_t* __restrict__ keys_in,
                                                              const uint32_t* __restrict__ vals_in,
                                                              uint32_t* __restrict__ keys_out,
                                                              uint32_t* __restrict__ vals_out, int64_t n, int shift,
                                                              int digit_bits, const int32_t* __restrict__ offsets,
                                                              int ntiles) {
  __shared__ int32_t s_wc[kRsWarps][256];
  __shared__ int32_t s_run[256];
  __shared__ int32_t s_goff[256];
  const int nd = 1 << digit_bits;
  const uint32_t mask = (uint32_t)nd - 1u;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < nd; d += kRsThreads) {
    s_run[d] = 0;
    s_goff[d] = offsets[(int64_t)d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) s_wc[w][d] = 0;
  }
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kRsRounds; ++r) {
    int64_t idx = base + (int64_t)r * kRsThreads + threadIdx.x;
    bool valid = idx < n;
    uint32_t key = valid ? keys_in[idx] : 0u;
    uint32_t val = valid ? vals_in[idx] : 0u;
    uint32_t d = (key >> shift) & mask;
    unsigned match_key = valid ? d : 0xffffffffu;
    unsigned peers = __match_any_sync(0xffffffffu, match_key);
    int rank = __popc(peers & lt_mask);
    bool leader = valid && (rank == 0);
    if (leader) s_wc[warp][d] = __popc(peers);
    __syncthreads();
    for (int dd = threadIdx.x; dd < nd; dd += kRsThreads) {
      int run = s_run[dd];
#pragma unroll
      for (int w = 0; w < kRsWarps; ++w) {
        int c = s_wc[w][dd];
        s_wc[w][dd] = run;
        run += c;
      }
      s_run[dd] = run;
    }
    __syncthreads();
    if (valid) {
      int dst = s_goff[d] + s_wc[warp][d] + rank;
      keys_out[dst] = key;
      vals_out[dst] = val;
    }
    __syncthreads();
    for (int dd = threadIdx.x; dd < nd; dd += kRsThreads) {
#pragma unroll
      for (int w = 0; w < kRsWarps; ++w) s_wc[w][dd] = 0;
    }
    __syncthreads();
  }
}

static int64_t rs_tiles(int64_t n) { return (n + kRsTile - 1) / kRsTile; }

}  // namespace sph

using namespace sph;

extern "C" {

int32_t sph_abi_version(void) { return 2; }

const char* sph_last_error(void) { return sph::g_err; }

const char* sph_status_string(sph_status_t s) {
  switch (s) {
    case SPH_OK: return "ok";
    case SPH_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SPH_ERR_CUDA: return "CUDA error";
    case SPH_ERR_SCRATCH_TOO_SMALL: return "scratch buffer too small";
    default: return "unknown status";
  }
}

uint64_t sph_scan_timeouts(void) {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_scan_timeouts, sizeof(v)) != cudaSuccess) return ~0ull;
  return v;
}

size_t sph_scan_scratch_bytes(int64_t n) { return (size_t)(scan_blocks(n < 1 ? 1 : n) + 2) * sizeof(int64_t); }

sph_status_t sph_exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch, size_t scratch_bytes,
                                    void* stream) {
  SPH_REQUIRE(n < (int64_t)1 << 31, "scan: n must be < 2^31 for int32 offsets");
  return scan_impl<int32_t>(in, out, n, scratch, scratch_bytes, stream);
}

sph_status_t sph_exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, void* scratch,
                                           size_t scratch_bytes, void* stream) {
  return scan_impl<int64_t>(in, out, n, scratch, scratch_bytes, stream);
}

int64_t sph_exclusive_scan_i32_static_max_items(void) {
  return (int64_t)(kStaticScanSlots - 1) * kScanTile;
}

sph_status_t sph_exclusive_scan_i32_static(const int32_t* in, int32_t* out, int64_t n, void* stream) {
  SPH_REQUIRE(n >= 0 && out != nullptr && (n == 0 || in != nullptr), "static scan: bad arguments");
  if (n > sph_exclusive_scan_i32_static_max_items()) {
    set_error_text("static scan: n exceeds the fixed scratch (at most 33,550,336 items); "
                   "use sph_exclusive_scan_i32 with caller-provided scratch");
    return SPH_ERR_INVALID_ARGUMENT;
  }
  void* scratch = nullptr;
  sph_status_t s = static_scan_scratch(&scratch);
  if (s != SPH_OK) return s;
  return scan_impl<int32_t>(in, out, n, scratch, sizeof(int64_t) * kStaticScanSlots, stream);
}

size_t sph_radix_sort_scratch_bytes(int64_t n, int32_t digit_bits) {
  if (digit_bits < 1) digit_bits = 1;
  if (digit_bits > 8) digit_bits = 8;
  int64_t nt = rs_tiles(n < 1 ? 1 : n);
  size_t hist = (size_t)(nt << digit_bits) + 1;
  size_t bytes = 2 * (size_t)n * sizeof(uint32_t);  // ping-pong keys + vals
  bytes += 2 * hist * sizeof(int32_t);              // histogram + scanned offsets
  bytes += sph_scan_scratch_bytes((int64_t)hist);
  return bytes + 256;
}

sph_status_t sph_radix_sort_pairs(uint32_t* keys, uint32_t* vals, int64_t n, int32_t key_bits, int32_t digit_bits,
                                  void* scratch, size_t scratch_bytes, void* stream) {
  SPH_REQUIRE(n >= 0 && n < ((int64_t)1 << 31), "radix sort: n out of range");
  SPH_REQUIRE(digit_bits >= 1 && digit_bits <= 8, "radix sort: digit_bits must be 1..8");
  SPH_REQUIRE(key_bits >= 0 && key_bits <= 32, "radix sort: key_bits must be 0..32");
  if (n <= 1 || key_bits == 0) return SPH_OK;
  if (scratch == nullptr || scratch_bytes < sph_radix_sort_scratch_bytes(n, digit_bits)) {
    set_error_text("radix sort: scratch too small");
    return SPH_ERR_SCRATCH_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  int64_t nt = rs_tiles(n);
  size_t hist_n = (size_t)(nt << digit_bits);
  char* p = reinterpret_cast<char*>(scratch);
  uint32_t* k_alt = reinterpret_cast<uint32_t*>(p);
  p += (size_t)n * sizeof(uint32_t);
  uint32_t* v_alt = reinterpret_cast<uint32_t*>(p);
  p += (size_t)n * sizeof(uint32_t);
  int32_t* hist = reinterpret_cast<int32_t*>(p);
  p += (hist_n + 1) * sizeof(int32_t);
  int32_t* offs = reinterpret_cast<int32_t*>(p);
  p += (hist_n + 1) * sizeof(int32_t);
  p = reinterpret_cast<char*>(((uintptr_t)p + 15) & ~(uintptr_t)15);
  void* scan_scratch = p;
  size_t scan_bytes = sph_scan_scratch_bytes((int64_t)hist_n + 1);

  int passes = (key_bits + digit_bits - 1) / digit_bits;
  uint32_t *kin = keys, *vin = vals, *kout = k_alt, *vout = v_alt;
  for (int pass = 0; pass < passes; ++pass) {
    int shift = pass * digit_bits;
    int bits = digit_bits;
    if (shift + bits > key_bits) bits = key_bits - shift;
    k_radix_hist<<<(unsigned)nt, kRsThreads, 0, st>>>(kin, n, shift, bits, hist, (int)nt);
    sph_status_t s = scan_impl<int32_t>(hist, offs, (int64_t)(nt << bits), scan_scratch, scan_bytes, stream);
    if (s != SPH_OK) return s;
    k_radix_scatter<<<(unsigned)nt, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, shift, bits, offs, (int)nt);
    SPH_CHECK_LAUNCH("radix sort pass");
    uint32_t* t = kin; kin = kout; kout = t;
    t = vin; vin = vout; vout = t;
  }
  if (kin != keys) {
    cudaMemcpyAsync(keys, kin, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(vals, vin, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    SPH_CHECK_LAUNCH("radix sort copy-back");
  }
  return SPH_OK;
}

}  // extern "C"
