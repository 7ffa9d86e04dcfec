// sort.cu — stable LSD radix sort of (key, u32 value) pairs, onesweep style
// (Adinets & Merrill, "Onesweep: A Faster Least Significant Digit Radix Sort
// for GPUs", 2022): one upfront histogram of every digit, then one kernel per
// 8-bit digit that ranks a tile with warp match/ballot operations, obtains its
// global offsets through a decoupled look-back over preceding tiles, and
// scatters through shared memory so that runs of equal digits are written
// contiguously.  Stability (equal keys keep ascending input position) is what
// makes the permutation equal to del-msh-cpu's `sort_by_key` over an iota
// (mortons.rs:139-146).
//
// The look-back waits on flags written by tiles that started earlier (tile
// ids are taken in launch order from an atomic counter), and every wait is
// bounded: after `spin_limit` polls (the process-wide wait limit, by default
// 2^22, read at each launch) the kernel raises kStatusSpinTimeout and carries
// on instead of hanging.
#include "dm_device.cuh"
#include "dm_internal.h"

namespace dm {
namespace {

constexpr int kThreads = 256;  // == kRadix: thread d owns digit d in the per-digit steps
constexpr int kWarps = kThreads / 32;
constexpr int kKpt = kSortTile / kThreads;  // keys per thread (15)
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
static_assert(kThreads == kRadix, "one thread per digit");
static_assert(kKpt * kThreads == kSortTile, "tile size");

template <typename KeyT>
__device__ __forceinline__ uint32_t digit_of(KeyT k, uint32_t shift) {
  return static_cast<uint32_t>(k >> shift) & (kRadix - 1);
}

// Exclusive scan of one value per thread over the 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp /* kWarps */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kWarps ? s_warp[lane] : 0u;
#pragma unroll
    for (int off = 1; off < kWarps; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    if (lane < kWarps) s_warp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const uint32_t before = warp > 0 ? s_warp[warp - 1] : 0u;
  const uint32_t r = before + x - v;
  __syncthreads();  // s_warp may be reused right after
  return r;
}

template <typename KeyT>
struct SortSmem {
  uint32_t whist[kWarps][kRadix];  // per-warp digit counts, then per-warp exclusive offsets
  uint32_t gbase[kRadix];          // global start of each digit (upfront histogram scan)
  uint32_t tstart[kRadix];         // start of each digit inside the tile
  uint32_t excl[kRadix];           // this tile's offset inside each digit (look-back)
  uint32_t scan[kWarps];
  uint32_t tile;
  KeyT keys[kSortTile];
  uint32_t vals[kSortTile];
};

template <typename KeyT, bool kIota, int kWindow>
__global__ void __launch_bounds__(kThreads, sizeof(KeyT) == 4 ? 4 : 2) k_onesweep(const KeyT* __restrict__ keys_in,
                                                      const uint32_t* __restrict__ vals_in, KeyT* __restrict__ keys_out,
                                                      uint32_t* __restrict__ vals_out, uint32_t n, uint32_t shift,
                                                      const uint32_t* __restrict__ hist, uint32_t* lookback,
                                                      uint32_t* tile_counter, uint32_t* status,
                                                      uint32_t spin_limit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortSmem<KeyT>& S = *reinterpret_cast<SortSmem<KeyT>*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int i = tid; i < kWarps * kRadix; i += kThreads) (&S.whist[0][0])[i] = 0u;
  // This pass's tile counter is zeroed before the sort starts and touched by
  // no other pass, so the ticket may be taken before the previous pass ends.
  if (tid == 0) S.tile = atomicAdd(tile_counter, 1u);
  pdl_wait();
  pdl_launch_dependents();
  const uint32_t gb = block_exclusive_scan(__ldg(hist + tid), S.scan);  // has __syncthreads
  S.gbase[tid] = gb;
  const uint32_t tile = S.tile;
  const uint32_t tile_base = tile * kSortTile;
  const uint32_t wbase = tile_base + static_cast<uint32_t>(warp) * 32u * kKpt;

  // Load the keys (warp-striped: key j of this lane is at wbase + 32*j + lane);
  // the values are loaded after ranking, to keep them out of its registers.
  KeyT keys[kKpt];
  uint32_t ranks[kKpt];
#pragma unroll
  for (int j = 0; j < kKpt; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    keys[j] = idx < n ? keys_in[idx] : KeyT{0};
  }

  // Rank inside the warp in (j, lane) order, i.e. input order.
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t* my_hist = S.whist[warp];
#pragma unroll
  for (int j = 0; j < kKpt; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    const bool valid = idx < n;
    const uint32_t d = digit_of(keys[j], shift);
    const uint32_t peers = warp_peers(d, valid);
    const uint32_t before = valid ? my_hist[d] : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) my_hist[d] = before + __popc(peers);
    __syncwarp();
    ranks[j] = before + __popc(peers & lt_mask);
  }
  uint32_t vals[kKpt];  // in flight while the counts are combined and scanned
#pragma unroll
  for (int j = 0; j < kKpt; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    vals[j] = kIota ? idx : (idx < n ? vals_in[idx] : 0u);
  }
  __syncthreads();

  // Thread d: per-warp exclusive offsets and the tile count of digit d.
  const uint32_t d = tid;
  uint32_t cnt = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) {
    const uint32_t c = S.whist[w][d];
    S.whist[w][d] = cnt;
    cnt += c;
  }
  // Publish this tile's count at once, so that successors looking back find it.
  volatile uint32_t* lb = lookback;
  if (tile == 0) lb[d] = kFlagInc | cnt;
  else lb[static_cast<size_t>(tile) * kRadix + d] = kFlagAgg | cnt;

  // The tile-local layout needs no global information: scatter the tile into
  // shared memory in (digit, input order) before looking back, so that the
  // keys, values and ranks no longer hold registers during the look-back.
  const uint32_t ts = block_exclusive_scan(cnt, S.scan);  // has __syncthreads
  S.tstart[d] = ts;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kKpt; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    if (idx < n) {
      const uint32_t dg = digit_of(keys[j], shift);
      const uint32_t pos = S.tstart[dg] + S.whist[warp][dg] + ranks[j];
      S.keys[pos] = keys[j];
      S.vals[pos] = vals[j];
    }
  }

  // Decoupled look-back for digit d: walk back over the predecessors kWindow
  // at a time (independent loads in flight together), consuming them in
  // order until an inclusive prefix.  Every tile publishes its count right
  // after ranking.  kWindow is a tuning choice (4 or 8); 4 measured fastest
  // on GB300 for 2M keys (105 us for four passes against 107 / 111 / 115 /
  // 132 us with 8 / 12 / 16 / 32): the inclusive prefix is usually a few
  // tiles back.
  uint32_t excl = 0;
  if (tile != 0) {
    int64_t k = static_cast<int64_t>(tile) - 1;
    uint32_t spins = 0;
    bool done = false;
    while (!done && k >= 0) {
      uint32_t v[kWindow];
#pragma unroll
      for (int j = 0; j < kWindow; ++j) {
        const uint32_t pad = kFlagInc;  // below tile 0: never consumed (tile 0 publishes an inclusive prefix)
        v[j] = (k - j >= 0) ? static_cast<uint32_t>(lb[static_cast<size_t>(k - j) * kRadix + d]) : pad;
      }
      bool stalled = false;
#pragma unroll
      for (int j = 0; j < kWindow; ++j) {
        if (done || stalled || k < 0) continue;
        const uint32_t flag = v[j] & ~kValueMask;
        if (flag == 0u) {
          stalled = true;  // predecessor k not published yet: re-read from k
          continue;
        }
        excl += v[j] & kValueMask;
        if (flag == kFlagInc) done = true;
        else --k;
      }
      if (stalled) {
        if (++spins > spin_limit) {
          raise_status(status, kStatusSpinTimeout);
          break;
        }
        __nanosleep(32);
      }
    }
    lb[static_cast<size_t>(tile) * kRadix + d] = kFlagInc | ((excl + cnt) & kValueMask);
  }
  S.excl[d] = excl;
  __syncthreads();

  // Write out: consecutive shared slots of one digit go to consecutive addresses.
  const uint32_t tile_n = (n - tile_base) < static_cast<uint32_t>(kSortTile) ? (n - tile_base) : kSortTile;
  for (uint32_t i = tid; i < tile_n; i += kThreads) {
    const KeyT k = S.keys[i];
    const uint32_t dg = digit_of(k, shift);
    const uint32_t g = S.gbase[dg] + S.excl[dg] + (i - S.tstart[dg]);
    if (g < n) {  // always true unless a look-back wait gave up (status already raised)
      keys_out[g] = k;
      vals_out[g] = S.vals[i];
    }
  }
}

// ------------------------------------------------------ match-ranked pass
// The 8-bit pass for u32 keys above kRadix10MaxKeys.  A tile is 4096 keys:
// 512 threads x 8 keys, warp-striped (key j of a lane at warp base + 32 j +
// lane, so (j, lane) order is input order).  A warp ranks a key by OR-ing its
// lane bit into the key's digit slot of a per-warp mask array in shared
// memory: after a __syncwarp the slot holds exactly the lanes with that digit
// (the peers), the lowest of them advances the warp's running count of the
// digit and clears the slot.  That is about 15 instructions per key against
// the ~40 of eight ballots, and with 8 keys per thread the pass keeps keys,
// ranks and values in registers without spilling.  Counts, look-back and
// write-out are those of k_onesweep.
constexpr int kThreadsM = 512;
constexpr int kWarpsM = kThreadsM / 32;
constexpr int kKptM = 8;
constexpr int kTileM = kThreadsM * kKptM;  // 4096
static_assert(kTileM >= kSortTile, "a match-pass tile covers at least a k_onesweep tile (look-back sizing)");

struct SortSmemM {
  uint32_t whist[kWarpsM][kRadix];  // per-warp running counts, then per-warp exclusive offsets
  uint32_t match[kWarpsM][kRadix];  // peer masks of the rank step; zero between steps
  uint32_t gbase[kRadix];           // global start of each digit (upfront histogram scan)
  uint32_t tstart[kRadix];          // start of each digit inside the tile
  uint32_t offs[kRadix];            // output position minus tile slot, per digit
  uint32_t scan[kWarpsM];
  uint32_t tile;
  uint32_t keys[kTileM];
  uint32_t vals[kTileM];
};

// Exclusive scan over the block of one value per thread (threads >= 256
// contribute zeros in the per-digit steps); has __syncthreads.
__device__ __forceinline__ uint32_t block_exclusive_scan_m(uint32_t v, uint32_t* s_warp /* kWarpsM */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kWarpsM ? s_warp[lane] : 0u;
#pragma unroll
    for (int off = 1; off < kWarpsM; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    if (lane < kWarpsM) s_warp[lane] = w;
  }
  __syncthreads();
  const uint32_t r = (warp > 0 ? s_warp[warp - 1] : 0u) + x - v;
  __syncthreads();
  return r;
}

template <bool kIota, int kWindow>
__global__ void __launch_bounds__(kThreadsM, 2) k_onesweep_match(const uint32_t* __restrict__ keys_in,
                                                               const uint32_t* __restrict__ vals_in,
                                                               uint32_t* __restrict__ keys_out,
                                                               uint32_t* __restrict__ vals_out, uint32_t n,
                                                               uint32_t shift, const uint32_t* __restrict__ hist,
                                                               uint32_t* lookback, uint32_t* tile_counter,
                                                               uint32_t* status, uint32_t spin_limit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortSmemM& S = *reinterpret_cast<SortSmemM*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  {
    uint4* z = reinterpret_cast<uint4*>(&S.whist[0][0]);  // whist and match: 2 * kWarpsM * kRadix words
    for (int i = tid; i < 2 * kWarpsM * kRadix / 4; i += kThreadsM) z[i] = make_uint4(0u, 0u, 0u, 0u);
  }
  // This pass's tile counter is zeroed before the sort starts and touched by
  // no other pass, so the ticket may be taken before the previous pass ends.
  if (tid == 0) S.tile = atomicAdd(tile_counter, 1u);
  pdl_wait();
  pdl_launch_dependents();
  const uint32_t gb = block_exclusive_scan_m(tid < kRadix ? __ldg(hist + tid) : 0u, S.scan);  // has __syncthreads
  if (tid < kRadix) S.gbase[tid] = gb;
  const uint32_t tile = S.tile;
  const uint32_t tile_base = tile * kTileM;
  const uint32_t wbase = tile_base + static_cast<uint32_t>(warp) * 32u * kKptM;

  uint32_t keys[kKptM], ranks[kKptM], vals[kKptM];
#pragma unroll
  for (int j = 0; j < kKptM; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    keys[j] = idx < n ? keys_in[idx] : 0u;
  }
#pragma unroll
  for (int j = 0; j < kKptM; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    vals[j] = kIota ? idx : (idx < n ? vals_in[idx] : 0u);
  }

  // Rank inside the warp in (j, lane) order, i.e. input order.
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t* wh = S.whist[warp];
  uint32_t* wm = S.match[warp];
#pragma unroll
  for (int j = 0; j < kKptM; ++j) {
    const bool valid = wbase + 32u * j + lane < n;
    const uint32_t d = (keys[j] >> shift) & (kRadix - 1);
    if (valid) atomicOr(wm + d, 1u << lane);
    __syncwarp();
    const uint32_t peers = valid ? wm[d] : 0u;
    const uint32_t before = valid ? wh[d] : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) {
      wh[d] = before + __popc(peers);
      wm[d] = 0u;
    }
    __syncwarp();
    ranks[j] = before + __popc(peers & lt_mask);
  }
  __syncthreads();

  // Thread d < 256: per-warp exclusive offsets and the tile count of digit d.
  const uint32_t d = tid;
  uint32_t cnt = 0;
  volatile uint32_t* lb = lookback;
  if (tid < kRadix) {
#pragma unroll
    for (int w = 0; w < kWarpsM; ++w) {
      const uint32_t c = S.whist[w][d];
      S.whist[w][d] = cnt;
      cnt += c;
    }
    // publish this tile's count at once, so that successors looking back find it
    if (tile == 0) lb[d] = kFlagInc | cnt;
    else lb[static_cast<size_t>(tile) * kRadix + d] = kFlagAgg | cnt;
  }
  const uint32_t ts = block_exclusive_scan_m(cnt, S.scan);  // has __syncthreads
  if (tid < kRadix) S.tstart[d] = ts;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kKptM; ++j) {
    if (wbase + 32u * j + lane < n) {
      const uint32_t dg = (keys[j] >> shift) & (kRadix - 1);
      const uint32_t pos = S.tstart[dg] + S.whist[warp][dg] + ranks[j];
      S.keys[pos] = keys[j];
      S.vals[pos] = vals[j];
    }
  }

  // Decoupled look-back for digit d (as k_onesweep).
  if (tid < kRadix) {
    uint32_t excl = 0;
    if (tile != 0) {
      int64_t k = static_cast<int64_t>(tile) - 1;
      uint32_t spins = 0;
      bool done = false;
      while (!done && k >= 0) {
        uint32_t v[kWindow];
#pragma unroll
        for (int j = 0; j < kWindow; ++j)
          v[j] = (k - j >= 0) ? static_cast<uint32_t>(lb[static_cast<size_t>(k - j) * kRadix + d]) : kFlagInc;
        bool stalled = false;
#pragma unroll
        for (int j = 0; j < kWindow; ++j) {
          if (done || stalled || k < 0) continue;
          const uint32_t flag = v[j] & ~kValueMask;
          if (flag == 0u) {
            stalled = true;  // predecessor k not published yet: re-read from k
            continue;
          }
          excl += v[j] & kValueMask;
          if (flag == kFlagInc) done = true;
          else --k;
        }
        if (stalled) {
          if (++spins > spin_limit) {
            raise_status(status, kStatusSpinTimeout);
            break;
          }
          __nanosleep(32);
        }
      }
      lb[static_cast<size_t>(tile) * kRadix + d] = kFlagInc | ((excl + cnt) & kValueMask);
    }
    // output position of tile slot i of digit d: base + excl + (i - tstart),
    // kept as one word (mod 2^32, so the subtraction may wrap)
    S.offs[d] = S.gbase[d] + excl - S.tstart[d];
  }
  __syncthreads();

  const uint32_t tile_n = (n - tile_base) < static_cast<uint32_t>(kTileM) ? (n - tile_base) : kTileM;
  for (uint32_t i = tid; i < tile_n; i += kThreadsM) {
    const uint32_t key = S.keys[i];
    const uint32_t g = S.offs[(key >> shift) & (kRadix - 1)] + i;
    if (g < n) {  // always true unless a look-back wait gave up (status already raised)
      keys_out[g] = key;
      vals_out[g] = S.vals[i];
    }
  }
}

template <int kWindow>
void onesweep_match_w(cudaStream_t s, uint32_t n, uint32_t shift, const uint32_t* keys_in, const uint32_t* vals_in,
                      uint32_t* keys_out, uint32_t* vals_out, const uint32_t* hist, uint32_t* lookback,
                      uint32_t* tile_counter, uint32_t* status, bool pdl) {
  const size_t smem = sizeof(SortSmemM);
  static bool configured[64] = {false};  // the attribute is per device and function
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    cudaFuncSetAttribute(k_onesweep_match<true, kWindow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    cudaFuncSetAttribute(k_onesweep_match<false, kWindow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    configured[dev] = true;
  }
  const uint32_t grid = (n + kTileM - 1) / kTileM;
  auto* kernel = vals_in == nullptr ? k_onesweep_match<true, kWindow> : k_onesweep_match<false, kWindow>;
  const uint32_t spin_limit = get_wait_limit();
  if (pdl)
    launch_pdl(kernel, dim3(grid), dim3(kThreadsM), smem, s, keys_in, vals_in, keys_out, vals_out, n, shift, hist,
               lookback, tile_counter, status, spin_limit);
  else
    kernel<<<grid, kThreadsM, smem, s>>>(keys_in, vals_in, keys_out, vals_out, n, shift, hist, lookback, tile_counter,
                                         status, spin_limit);
}

// ---------------------------------------------------------------- 10-bit
// The same pass over a 10-bit digit of u32 keys (1024 digits), so that three
// passes sort 30-bit Morton codes.  Each thread owns 4 consecutive digits in
// the per-digit steps; the per-warp counts are 16-bit (a warp ranks at most
// 32 * kKpt = 480 keys) and the look-back result is folded with the global
// base into one offset per digit, which keeps a tile at ~54 KB of shared
// memory (four tiles per SM, as the 8-bit pass).
constexpr int kDpt10 = kRadix10 / kThreads;  // digits per thread: 4
static_assert(kDpt10 == 4, "four digits per thread");

struct SortSmem10 {
  uint16_t whist[kWarps][kRadix10];  // per-warp digit counts, then per-warp exclusive offsets
  uint32_t tstart[kRadix10];         // start of each digit inside the tile
  uint32_t offs[kRadix10];           // global base, then output position minus tile slot
  uint32_t scan[kWarps];
  uint32_t tile;
  uint32_t keys[kSortTile];
  uint32_t vals[kSortTile];
};

__device__ __forceinline__ uint32_t digit10(uint32_t k, uint32_t shift) { return (k >> shift) & (kRadix10 - 1); }

__device__ __forceinline__ uint32_t warp_peers10(uint32_t d, bool valid) {
  uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < 10; ++b) {
    const bool bit = (d >> b) & 1u;
    const uint32_t bb = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? bb : ~bb;
  }
  return peers;
}

template <bool kIota, int kWindow>
__global__ void __launch_bounds__(kThreads, 4) k_onesweep10(const uint32_t* __restrict__ keys_in,
                                                          const uint32_t* __restrict__ vals_in,
                                                          uint32_t* __restrict__ keys_out,
                                                          uint32_t* __restrict__ vals_out, uint32_t n, uint32_t shift,
                                                          const uint32_t* __restrict__ hist, uint32_t* lookback,
                                                          uint32_t* tile_counter, uint32_t* status,
                                                          uint32_t spin_limit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortSmem10& S = *reinterpret_cast<SortSmem10*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  {
    uint32_t* w = reinterpret_cast<uint32_t*>(&S.whist[0][0]);
    for (int i = tid; i < kWarps * kRadix10 / 2; i += kThreads) w[i] = 0u;
  }
  // This pass's tile counter is zeroed before the sort starts and touched by
  // no other pass, so the ticket may be taken before the previous pass ends.
  if (tid == 0) S.tile = atomicAdd(tile_counter, 1u);
  pdl_wait();
  pdl_launch_dependents();
  // global start of digits 4*tid .. 4*tid+3 (scan of the upfront histogram)
  const uint4 h4 = __ldg(reinterpret_cast<const uint4*>(hist) + tid);
  const uint32_t hsum = h4.x + h4.y + h4.z + h4.w;
  {
    const uint32_t base = block_exclusive_scan(hsum, S.scan);  // has __syncthreads
    S.offs[4 * tid] = base;
    S.offs[4 * tid + 1] = base + h4.x;
    S.offs[4 * tid + 2] = base + h4.x + h4.y;
    S.offs[4 * tid + 3] = base + h4.x + h4.y + h4.z;
  }
  const uint32_t tile = S.tile;
  const uint32_t tile_base = tile * kSortTile;
  const uint32_t wbase = tile_base + static_cast<uint32_t>(warp) * 32u * kKpt;

  uint32_t keys[kKpt];
  uint32_t ranks[kKpt];
#pragma unroll
  for (int j = 0; j < kKpt; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    keys[j] = idx < n ? keys_in[idx] : 0u;
  }
  // Rank inside the warp in (j, lane) order, i.e. input order.
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint16_t* my_hist = S.whist[warp];
#pragma unroll
  for (int j = 0; j < kKpt; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    const bool valid = idx < n;
    const uint32_t d = digit10(keys[j], shift);
    const uint32_t peers = warp_peers10(d, valid);
    const uint32_t before = valid ? my_hist[d] : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) my_hist[d] = static_cast<uint16_t>(before + __popc(peers));
    __syncwarp();
    ranks[j] = before + __popc(peers & lt_mask);
  }
  __syncthreads();

  // Digits 4*tid+q: per-warp exclusive offsets and the tile counts.
  uint32_t cnt[kDpt10];
#pragma unroll
  for (int q = 0; q < kDpt10; ++q) {
    const uint32_t d = 4 * tid + q;
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      const uint32_t x = S.whist[w][d];
      S.whist[w][d] = static_cast<uint16_t>(c);
      c += x;
    }
    cnt[q] = c;
  }
  // Publish this tile's counts at once, so that successors looking back find them.
  volatile uint32_t* lb = lookback + static_cast<size_t>(tile) * kRadix10 + 4 * tid;
  const uint32_t pflag = tile == 0 ? kFlagInc : kFlagAgg;
#pragma unroll
  for (int q = 0; q < kDpt10; ++q) lb[q] = pflag | cnt[q];

  // Tile-local layout, then the scatter into shared memory (as the 8-bit pass).
  {
    const uint32_t csum = cnt[0] + cnt[1] + cnt[2] + cnt[3];
    const uint32_t ts = block_exclusive_scan(csum, S.scan);  // has __syncthreads
    S.tstart[4 * tid] = ts;
    S.tstart[4 * tid + 1] = ts + cnt[0];
    S.tstart[4 * tid + 2] = ts + cnt[0] + cnt[1];
    S.tstart[4 * tid + 3] = ts + cnt[0] + cnt[1] + cnt[2];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kKpt; ++j) {
    const uint32_t idx = wbase + 32u * j + lane;
    if (idx < n) {
      const uint32_t dg = digit10(keys[j], shift);
      const uint32_t pos = S.tstart[dg] + S.whist[warp][dg] + ranks[j];
      S.keys[pos] = keys[j];
      S.vals[pos] = kIota ? idx : vals_in[idx];
    }
  }

  // Decoupled look-back for the thread's 4 digits together: predecessor k's 4
  // words are read as one uint4; a round reads kWindow predecessors and
  // consumes them in order until every digit has met an inclusive prefix.
  uint32_t excl[kDpt10] = {0u, 0u, 0u, 0u};
  if (tile != 0) {
    bool done[kDpt10] = {false, false, false, false};
    int64_t k = static_cast<int64_t>(tile) - 1;
    uint32_t spins = 0;
    const volatile uint4* lb4 = reinterpret_cast<const volatile uint4*>(lookback) + tid;  // + kRadix10/4 per tile
    bool all_done = false;
    while (!all_done && k >= 0) {
      uint4 v[kWindow];
#pragma unroll
      for (int j = 0; j < kWindow; ++j) {
        if (k - j >= 0) {
          const volatile uint4* p = lb4 + static_cast<size_t>(k - j) * (kRadix10 / 4);
          v[j] = make_uint4(p->x, p->y, p->z, p->w);
        } else {
          v[j] = make_uint4(kFlagInc, kFlagInc, kFlagInc, kFlagInc);  // below tile 0: never consumed
        }
      }
      bool stalled = false;
#pragma unroll
      for (int j = 0; j < kWindow; ++j) {
        if (all_done || stalled || k < 0) continue;
        const uint32_t w4[4] = {v[j].x, v[j].y, v[j].z, v[j].w};
        bool ready = true;
#pragma unroll
        for (int q = 0; q < kDpt10; ++q) ready = ready && (done[q] || (w4[q] & ~kValueMask) != 0u);
        if (!ready) {
          stalled = true;  // predecessor k not fully published yet: re-read from k
          continue;
        }
        all_done = true;
#pragma unroll
        for (int q = 0; q < kDpt10; ++q) {
          if (done[q]) continue;
          excl[q] += w4[q] & kValueMask;
          if ((w4[q] & ~kValueMask) == kFlagInc) done[q] = true;
          all_done = all_done && done[q];
        }
        --k;
      }
      if (stalled) {
        if (++spins > spin_limit) {
          raise_status(status, kStatusSpinTimeout);
          break;
        }
        __nanosleep(32);
      }
    }
#pragma unroll
    for (int q = 0; q < kDpt10; ++q) lb[q] = kFlagInc | ((excl[q] + cnt[q]) & kValueMask);
  }
  // output position of tile slot i of digit d: base + excl + (i - tstart),
  // kept as one word (mod 2^32, so the subtraction may wrap)
#pragma unroll
  for (int q = 0; q < kDpt10; ++q) {
    const uint32_t d = 4 * tid + q;
    S.offs[d] = S.offs[d] + excl[q] - S.tstart[d];
  }
  __syncthreads();

  const uint32_t tile_n = (n - tile_base) < static_cast<uint32_t>(kSortTile) ? (n - tile_base) : kSortTile;
  for (uint32_t i = tid; i < tile_n; i += kThreads) {
    const uint32_t key = S.keys[i];
    const uint32_t g = S.offs[digit10(key, shift)] + i;
    if (g < n) {  // always true unless a look-back wait gave up (status already raised)
      keys_out[g] = key;
      vals_out[g] = S.vals[i];
    }
  }
}

template <int kWindow>
void onesweep10_w(cudaStream_t s, uint32_t n, uint32_t shift, const uint32_t* keys_in, const uint32_t* vals_in,
                  uint32_t* keys_out, uint32_t* vals_out, const uint32_t* hist, uint32_t* lookback,
                  uint32_t* tile_counter, uint32_t* status) {
  const size_t smem = sizeof(SortSmem10);
  static bool configured[64] = {false};  // the attribute is per device and function
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    cudaFuncSetAttribute(k_onesweep10<true, kWindow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    cudaFuncSetAttribute(k_onesweep10<false, kWindow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    configured[dev] = true;
  }
  auto* kernel = vals_in == nullptr ? k_onesweep10<true, kWindow> : k_onesweep10<false, kWindow>;
  launch_pdl(kernel, dim3(sort_num_tiles(n)), dim3(kThreads), smem, s, keys_in, vals_in, keys_out, vals_out, n, shift,
             hist, lookback, tile_counter, status, get_wait_limit());
}

template <typename KeyT>
__global__ void __launch_bounds__(kThreads) k_digit_hist(uint32_t n, const KeyT* __restrict__ keys, int num_pass,
                                                        uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[8 * kRadix];
  for (int i = threadIdx.x; i < num_pass * kRadix; i += kThreads) sh[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const KeyT k = keys[i];
    for (int p = 0; p < num_pass; ++p) atomicAdd(&sh[p * kRadix + digit_of(k, 8u * p)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < num_pass * kRadix; i += kThreads)
    if (sh[i]) atomicAdd(hist + i, sh[i]);
}

template <typename KeyT, int kWindow>
void onesweep_w(cudaStream_t s, uint32_t n, uint32_t shift, const KeyT* keys_in, const uint32_t* vals_in,
                KeyT* keys_out, uint32_t* vals_out, const uint32_t* hist, uint32_t* lookback, uint32_t* tile_counter,
                uint32_t* status, bool pdl) {
  const size_t smem = sizeof(SortSmem<KeyT>);
  static bool configured[64] = {false};  // the attribute is per device and function
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    cudaFuncSetAttribute(k_onesweep<KeyT, true, kWindow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    cudaFuncSetAttribute(k_onesweep<KeyT, false, kWindow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    configured[dev] = true;
  }
  const uint32_t grid = sort_num_tiles(n);
  auto* kernel = vals_in == nullptr ? k_onesweep<KeyT, true, kWindow> : k_onesweep<KeyT, false, kWindow>;
  const uint32_t spin_limit = get_wait_limit();
  if (pdl)
    launch_pdl(kernel, dim3(grid), dim3(kThreads), smem, s, keys_in, vals_in, keys_out, vals_out, n, shift, hist,
               lookback, tile_counter, status, spin_limit);
  else
    kernel<<<grid, kThreads, smem, s>>>(keys_in, vals_in, keys_out, vals_out, n, shift, hist, lookback, tile_counter,
                                        status, spin_limit);
}

template <typename KeyT>
void onesweep(cudaStream_t s, uint32_t n, uint32_t shift, const KeyT* keys_in, const uint32_t* vals_in,
              KeyT* keys_out, uint32_t* vals_out, const uint32_t* hist, uint32_t* lookback, uint32_t* tile_counter,
              uint32_t* status, bool pdl) {
  if (n == 0) return;
  if (get_tuning().sort_window == 8)
    onesweep_w<KeyT, 8>(s, n, shift, keys_in, vals_in, keys_out, vals_out, hist, lookback, tile_counter, status, pdl);
  else
    onesweep_w<KeyT, 4>(s, n, shift, keys_in, vals_in, keys_out, vals_out, hist, lookback, tile_counter, status, pdl);
}

}  // namespace

void launch_digit_hist_u32(cudaStream_t s, uint32_t n, const uint32_t* keys, int num_pass, uint32_t* hist) {
  uint32_t grid = (n + kThreads * 16 - 1) / (kThreads * 16);
  if (grid < 1) grid = 1;
  if (grid > 152 * 8) grid = 152 * 8;
  k_digit_hist<uint32_t><<<grid, kThreads, 0, s>>>(n, keys, num_pass, hist);
}

void launch_digit_hist_u64(cudaStream_t s, uint32_t n, const uint64_t* keys, int num_pass, uint32_t* hist) {
  uint32_t grid = (n + kThreads * 16 - 1) / (kThreads * 16);
  if (grid < 1) grid = 1;
  if (grid > 152 * 8) grid = 152 * 8;
  k_digit_hist<uint64_t><<<grid, kThreads, 0, s>>>(n, keys, num_pass, hist);
}

void launch_onesweep_u32(cudaStream_t s, uint32_t n, uint32_t shift, const uint32_t* keys_in,
                         const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, const uint32_t* hist,
                         uint32_t* lookback, uint32_t* tile_counter, uint32_t* status, bool pdl) {
  if (n == 0) return;
  if (get_tuning().sort_window == 8)
    onesweep_match_w<8>(s, n, shift, keys_in, vals_in, keys_out, vals_out, hist, lookback, tile_counter, status, pdl);
  else
    onesweep_match_w<4>(s, n, shift, keys_in, vals_in, keys_out, vals_out, hist, lookback, tile_counter, status, pdl);
}

void launch_onesweep10_u32(cudaStream_t s, uint32_t n, uint32_t shift, const uint32_t* keys_in,
                           const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, const uint32_t* hist,
                           uint32_t* lookback, uint32_t* tile_counter, uint32_t* status) {
  if (n == 0) return;
  if (get_tuning().sort_window == 8)
    onesweep10_w<8>(s, n, shift, keys_in, vals_in, keys_out, vals_out, hist, lookback, tile_counter, status);
  else
    onesweep10_w<4>(s, n, shift, keys_in, vals_in, keys_out, vals_out, hist, lookback, tile_counter, status);
}

void launch_onesweep_u64(cudaStream_t s, uint32_t n, uint32_t shift, const uint64_t* keys_in,
                         const uint32_t* vals_in, uint64_t* keys_out, uint32_t* vals_out, const uint32_t* hist,
                         uint32_t* lookback, uint32_t* tile_counter, uint32_t* status) {
  onesweep<uint64_t>(s, n, shift, keys_in, vals_in, keys_out, vals_out, hist, lookback, tile_counter, status, false);
}

// One 8-bit pass over a single tile of n <= kSortTile keys, launched as one
// block with the tile counter preset by the caller.  With the counter at 1
// the block draws tile 1 (beyond the keys: it loads and writes none) and its
// look-back waits for tile 0, which no block publishes, until `spin_limit`
// polls have passed.  Used only to check that a wait that never ends gives
// up, raises kStatusSpinTimeout and returns.
void launch_onesweep_wait_probe(cudaStream_t s, uint32_t n, const uint32_t* keys_in, uint32_t* keys_out,
                                uint32_t* vals_out, const uint32_t* hist, uint32_t* lookback, uint32_t* tile_counter,
                                uint32_t* status, uint32_t spin_limit) {
  const size_t smem = sizeof(SortSmem<uint32_t>);
  cudaFuncSetAttribute(k_onesweep<uint32_t, true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(smem));
  k_onesweep<uint32_t, true, 4><<<1, kThreads, smem, s>>>(keys_in, nullptr, keys_out, vals_out, n, 0u, hist,
                                                          lookback, tile_counter, status, spin_limit);
}

}  // namespace dm
